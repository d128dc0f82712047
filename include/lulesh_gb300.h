/*
 * lulesh_gb300.h - C ABI of the GB300 (sm_103a) LagrangeLeapFrog library.
 *
 * Drop-in for the single-rank timestep of JuliaLabs/LULESH.jl. A handle owns
 * one Sedov problem whose nodal and element fields live on the GPU as FP64
 * structure-of-arrays buffers; the host only sees the step's scalars unless it
 * asks for a field. Every entry point returns a lulesh_status code (0 = OK).
 *
 * Plain C types only: a Julia `ccall`, a Python ctypes stub or C/C++ code can
 * bind it directly. One handle is driven by one host thread at a time.
 */
#ifndef LULESH_GB300_H
#define LULESH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The reference raises Julia exceptions at the same points. */
typedef enum {
  LULESH_OK = 0,
  LULESH_ERR_VOLUME = 1,     /* any "Volume Error" (src/domain.jl:1104,1727,1758,2118,2169,2905,2926) */
  LULESH_ERR_QSTOP = 2,      /* "QStopError" (src/domain.jl:2580) */
  LULESH_ERR_BAD_BC = 3,     /* error("Error") on an invalid elemBC mask (src/domain.jl:2343) */
  LULESH_ERR_CUDA = 4,       /* a CUDA runtime call failed */
  LULESH_ERR_TIMEOUT = 5,    /* a bounded device wait ran out */
  LULESH_ERR_ARGUMENT = 6,   /* bad argument (null pointer, unknown id, size mismatch) */
  LULESH_ERR_MEMORY = 7,     /* device allocation failed */
  LULESH_ERR_INDEX = 8       /* a build with -DLULESH_CHECK met an index outside its range
                                (the access was skipped); never raised by a normal build */
} lulesh_status;

/* Which reference check raised a LULESH_ERR_VOLUME (finer than the code). */
typedef enum {
  LULESH_SITE_NONE = 0,
  LULESH_SITE_EARLY = 1,       /* integrateStressForElems, src/domain.jl:1104 */
  LULESH_SITE_HOURGLASS = 2,   /* calcHourglassControlForElems, src/domain.jl:1727 */
  LULESH_SITE_MID = 3,         /* calcVolumeForceForElems, src/domain.jl:1758 */
  LULESH_SITE_KINEMATICS = 4,  /* calcKinematicsForElems, src/domain.jl:2118 */
  LULESH_SITE_LAGRANGE = 5,    /* calcLagrangeElements, src/domain.jl:2169 */
  LULESH_SITE_MATERIAL = 6,    /* applyMaterialPropertiesForElems, src/domain.jl:2905 */
  LULESH_SITE_UPDATE = 7       /* updateVolumesForElems, src/domain.jl:2926 */
} lulesh_site;

/* Mode bits: 0 reproduces the reference exactly (including three defects of
 * its restatement); each bit corrects one of them. 7 = LULESH 2.0 method. */
enum {
  LULESH_MODE_FAITHFUL = 0,
  LULESH_FIX_NORMALS = 1,   /* calcElemNodeNormals face 5, src/domain.jl:1046-1055 */
  LULESH_FIX_VOLUDER = 2,   /* calcElemVolumeDerivative node slots, src/domain.jl:1253-1255 */
  LULESH_FIX_LXIP = 4,      /* xi-plus neighbour index, src/domain.jl:2349 */
  LULESH_MODE_LULESH2 = 7
};

/* Problem description: LuleshProblem (src/LULESH.jl:31-49) for one rank. */
typedef struct {
  int32_t nx;             /* elements per edge (>= 1) */
  int32_t nr;             /* regions (>= 1); src/domain.jl:338 */
  int32_t balance;        /* region balance exponent */
  int32_t cost;           /* region cost factor */
  int32_t mode;           /* LULESH_MODE_* bits */
  int32_t region_reps;    /* 0: regions cost nothing (the reference); 1: evaluate the
                             EOS regReps[r] times per region r (LULESH 2.0 cost model;
                             results are unchanged) */
  int32_t keep_aux;       /* 1: also store fx,fy,fz,xdd,ydd,zdd,dxx,dyy,dzz,ql,qq each
                             step, which the reference keeps in its Domain */
  int32_t device;         /* CUDA device ordinal */
  uint64_t region_seed;   /* seed of the region generator (Random.seed!(myRank)) */
} lulesh_params;

/* The Domain scalars that change every step (src/types.jl:98-107). */
typedef struct {
  double time;            /* domain.time */
  double deltatime;       /* domain.deltatime */
  double dtcourant;       /* domain.dtcourant */
  double dthydro;         /* domain.dthydro */
  int64_t cycle;          /* domain.cycle */
  int32_t status;         /* lulesh_status of the last step */
  int32_t site;           /* lulesh_site of the last LULESH_ERR_VOLUME */
} lulesh_scalars;

/* Field identifiers: the Domain vectors of src/types.jl:1-87. Double fields
 * are FP64; index fields are int64 holding the raw values the Julia Domain
 * stores; LULESH_F_ELEMBC is uint32. */
typedef enum {
  /* element-centred FP64 (numElem) */
  LULESH_F_E = 0, LULESH_F_P, LULESH_F_Q, LULESH_F_QL, LULESH_F_QQ, LULESH_F_V, LULESH_F_VOLO,
  LULESH_F_DELV, LULESH_F_VDOV, LULESH_F_AREALG, LULESH_F_SS, LULESH_F_ELEMMASS, LULESH_F_VNEW,
  LULESH_F_DELV_XI, LULESH_F_DELV_ETA, LULESH_F_DELV_ZETA, LULESH_F_DELX_XI, LULESH_F_DELX_ETA,
  LULESH_F_DELX_ZETA, LULESH_F_DXX, LULESH_F_DYY, LULESH_F_DZZ,
  /* node-centred FP64 (numNode) */
  LULESH_F_X = 32, LULESH_F_Y, LULESH_F_Z, LULESH_F_XD, LULESH_F_YD, LULESH_F_ZD, LULESH_F_XDD,
  LULESH_F_YDD, LULESH_F_ZDD, LULESH_F_FX, LULESH_F_FY, LULESH_F_FZ, LULESH_F_NODALMASS,
  /* int64 index fields (raw Julia values) */
  LULESH_F_NODELIST = 64,       /* 8*numElem, 0-based node ids, element-major */
  LULESH_F_LXIM, LULESH_F_LXIP, LULESH_F_LETAM, LULESH_F_LETAP, LULESH_F_LZETAM, LULESH_F_LZETAP,
  LULESH_F_SYMMX, LULESH_F_SYMMY, LULESH_F_SYMMZ,
  LULESH_F_NODEELEMCOUNT, LULESH_F_NODEELEMSTART, LULESH_F_NODEELEMCORNERLIST,
  LULESH_F_MATELEMLIST, LULESH_F_REGNUMLIST, LULESH_F_REGELEMLIST, LULESH_F_REGCSR,
  LULESH_F_REGREPS, LULESH_F_REGSORTED, LULESH_F_REGELEMSIZE,
  /* uint32 */
  LULESH_F_ELEMBC = 96
} lulesh_field;

/* Scalar identifiers: the Domain parameters of src/types.jl:91-126. */
typedef enum {
  LULESH_S_DTFIXED = 0, LULESH_S_DELTATIMEMULTLB, LULESH_S_DELTATIMEMULTUB, LULESH_S_STOPTIME,
  LULESH_S_DTMAX, LULESH_S_DTHYDRO, LULESH_S_DTCOURANT, LULESH_S_TIME, LULESH_S_DELTATIME,
  LULESH_S_U_CUT, LULESH_S_HGCOEF, LULESH_S_QSTOP, LULESH_S_MONOQ_MAX_SLOPE,
  LULESH_S_MONOQ_LIMITER_MULT, LULESH_S_E_CUT, LULESH_S_P_CUT, LULESH_S_SS4O3, LULESH_S_Q_CUT,
  LULESH_S_V_CUT, LULESH_S_QLC_MONOQ, LULESH_S_QQC_MONOQ, LULESH_S_QQC, LULESH_S_EOSVMAX,
  LULESH_S_EOSVMIN, LULESH_S_PMIN, LULESH_S_EMIN, LULESH_S_DVOVMAX, LULESH_S_REFDENS,
  LULESH_S_CYCLE, LULESH_S_COUNT
} lulesh_scalar;

typedef struct lulesh_domain lulesh_domain;

/* Fill *p with the reference defaults for an nx^3 problem (nr = 11 as the
 * reference's TODO asks, balance = cost = 1, mode 0). */
void lulesh_default_params(lulesh_params* p, int32_t nx);

/* Domain(prob): builds the Sedov mesh, connectivity, boundary conditions,
 * masses, energy deposit, initial dt and regions on the device.
 * Replaces Domain(prob::LuleshProblem), src/domain.jl:467-771. */
int lulesh_create(const lulesh_params* params, lulesh_domain** out);

/* Releases every device and host resource of the handle. */
int lulesh_destroy(lulesh_domain* dom);

/* timeIncrement!(domain): host-side dt control, src/domain.jl:920-961. */
int lulesh_time_increment(lulesh_domain* dom);

/* lagrangeLeapFrog(domain): one step on the device, src/domain.jl:3067-3080.
 * Copies the scalars in, runs the step kernels, copies dtcourant, dthydro and
 * the status back. Returns the step status. */
int lulesh_lagrange_leapfrog(lulesh_domain* dom);

/* The examples/benchmark.jl:82-98 loop (timeIncrement! then lagrangeLeapFrog
 * until time >= stoptime, stopping once cycle >= num_iters) run entirely on
 * the device from a captured CUDA graph; dt is computed on the device.
 * On return *out (if non-null) holds the final scalars. */
int lulesh_run(lulesh_domain* dom, int64_t num_iters, lulesh_scalars* out);

/* Current step scalars (time, deltatime, dtcourant, dthydro, cycle, status). */
int lulesh_get_scalars(const lulesh_domain* dom, lulesh_scalars* out);

/* Read / write one Domain scalar (getfield / setfield! on the Domain). */
int lulesh_get_scalar(const lulesh_domain* dom, int32_t id, double* value);
int lulesh_set_scalar(lulesh_domain* dom, int32_t id, double value);

/* Number of entries of a field (numElem, numNode, 8*numElem, ...). */
int lulesh_field_length(const lulesh_domain* dom, int32_t field, int64_t* count);

/* Copy a field between the device and a caller-owned host buffer of exactly
 * `count` entries (double, int64 or uint32 per the field). Synchronous. */
int lulesh_download_field(lulesh_domain* dom, int32_t field, void* host, int64_t count);
int lulesh_upload_field(lulesh_domain* dom, int32_t field, const void* host, int64_t count);

/* verifyAndWriteFinalOutput's numbers (src/utils.jl:124-158): out[0] = e[1]
 * (origin energy), out[1] = MaxAbsDiff, out[2] = TotalAbsDiff,
 * out[3] = MaxRelDiff of the plane-0 symmetry check. */
int lulesh_verify(lulesh_domain* dom, double out[4]);

/* Full-state files. The reference has no checkpoint format; these write the
 * handle's step state (x y z xd yd zd e p q v ss and every Domain scalar,
 * cycle included) to a binary file with a header naming the problem
 * (nx, nr, balance, cost, mode, sizes) and a trailing 64-bit FNV-1a hash, and
 * load it into a handle of the same problem, which then continues exactly as
 * the saved run would have. Loading checks the header and the hash before it
 * changes anything; a mismatch or a short file returns LULESH_ERR_ARGUMENT.
 * Format: lulesh.jl_gb300/csrc/lulesh_state_io.cu. */
int lulesh_save_state(lulesh_domain* dom, const char* path);
int lulesh_load_state(lulesh_domain* dom, const char* path);

/* numElem and numNode of the handle. */
int lulesh_sizes(const lulesh_domain* dom, int64_t* num_elem, int64_t* num_node);

/* The CUDA stream (cudaStream_t) the handle launches on, for callers that
 * order their own work or CUDA events against the step. */
int lulesh_get_stream(lulesh_domain* dom, void** stream);

/* Kernel timing: when enabled, each step records CUDA events around every
 * kernel on the handle's stream; lulesh_kernel_times returns the summed
 * milliseconds per kernel (names in the same order) and resets them. */
int lulesh_enable_timing(lulesh_domain* dom, int32_t enable);
int lulesh_kernel_times(lulesh_domain* dom, double* ms, int32_t max_kernels, int32_t* n_kernels);
const char* lulesh_kernel_name(int32_t index);

/* ---- Blocks of one mesh (the multi-rank decomposition) --------------------
 * The reference's multi-rank run splits the (tp*nx)^3 Sedov mesh into a cube
 * of tp^3 ranks of nx^3 elements each (initMeshDecomp, src/LULESH.jl:62-97)
 * and exchanges block-face data every cycle: the summed nodal forces
 * (commSBN, src/comm.jl:776), positions and velocities (commSyncPosVel,
 * src/comm.jl:1251), the monotonic-Q gradients beside a face (commMonoQ,
 * src/comm.jl:1127) and the time-step minimum (comm_min, src/mpi.jl:81).
 * lulesh_create_blocks builds that decomposition in one GPU's memory: the
 * handle's arrays hold the blocks one after another (rank order, each in its
 * per-rank element and node order, nodes on block faces once per block that
 * touches them; params->nx is the block edge), and every value that crosses
 * a block face is a ghost slot filled by a halo copy from the block that
 * owns it. The result is bitwise the single-block run of the whole mesh.
 * Every other call (step, run, fields, state files, tuning) works on the
 * packed arrays; lulesh_block_map gives each packed element's and node's id
 * in the whole mesh. Each block holds its rank's region sets (draws seeded
 * with region_seed + rank, numbers rotated by the rank; the nr-sized region
 * arrays a field download returns are rank 0's), so the region cost model
 * works on a block mesh; the adjoint needs one block.
 * lulesh_block_plan_sizes / lulesh_block_plan return the decomposition and
 * its halo plan without a GPU: per ghost slot the packed element (delv) or
 * corner-force slot c*E + e (corners) it copies and the block it belongs to;
 * sizes = {E, N, ghost delv slots, ghost corner slots, corner-list entries}. */
int lulesh_create_blocks(const lulesh_params* params, int32_t blocks_per_edge, lulesh_domain** out);
int lulesh_block_map(const lulesh_domain* dom, int32_t* blocks_per_edge, int32_t* elem_global,
                     int32_t* node_global);
int lulesh_block_plan_sizes(int32_t nx, int32_t blocks_per_edge, int32_t mode, int64_t sizes[5]);
int lulesh_block_plan(int32_t nx, int32_t blocks_per_edge, int32_t mode, int32_t* elem_global, int32_t* node_global,
                      int32_t* halo_delv_src, int32_t* halo_delv_dst, int32_t* halo_corner_src,
                      int32_t* halo_corner_dst);

/* ---- Launch tuning --------------------------------------------------------
 * Threads per block of the four step kernels and the fusion split of the
 * force geometry. lulesh_autotune tries each block-size candidate for one
 * kernel at a time on the live problem (cycles timed with CUDA events),
 * keeps the fastest, then times the other geometry split with its own best
 * force and kinematics blocks and keeps the faster split; it restores the
 * problem's state. No choice changes any result (bitwise). */
typedef struct {
  int32_t force_block;   /* k_force: 64, 128 or 256 */
  int32_t node_block;    /* k_node: 128, 256 or 512 */
  int32_t kin_block;     /* k_kinematics: 64, 128 or 256 */
  int32_t mat_block;     /* k_material: 64, 128 or 256 */
  int32_t geometry;      /* where the force kernel's geometry of the positions
                            (volume derivatives, hourglass modes, node normals)
                            is formed: 0 by k_kinematics of the cycle before,
                            stored (408 B per element); 1 inside k_force */
} lulesh_tuning;

int lulesh_get_tuning(const lulesh_domain* dom, lulesh_tuning* out);
int lulesh_set_tuning(lulesh_domain* dom, const lulesh_tuning* t);
int lulesh_autotune(lulesh_domain* dom, int32_t cycles, lulesh_tuning* chosen);

/* ---- Batched ensemble -------------------------------------------------------
 * Many independent single-rank Sedov problems advanced together: all
 * instances' elements and nodes are packed into one index space, so every
 * kernel launch covers every instance whatever their sizes; each instance
 * keeps its own dt, time, cycle and status, computed on the device. A run is
 * one launch of a CUDA graph of the whole run (runs over 512 cycles relaunch
 * it) with no host work per cycle. The
 * reference has one problem per process; this batches Domain(prob) /
 * timeIncrement! / lagrangeLeapFrog over instances. */
typedef struct {
  int32_t nx, nr, balance, cost;
  double einit;           /* energy deposited in the origin element; 0 = 3.948746e7*(nx/45)^3 */
  double hgcoef;          /* hourglass coefficient (the reference's default is 3.0) */
  uint64_t region_seed;
} lulesh_instance;

typedef struct lulesh_ensemble lulesh_ensemble;

/* Seeded instance draw (std::mt19937_64(seed)): nx uniform in [nx_min, nx_max],
 * einit = the default for nx times exp(U[ln 0.5, ln 2]), hgcoef uniform in
 * [2, 4], nr = 1 or 11 with probability 1/2 each, balance = cost = 1. */
int lulesh_ens_sedov_instances(uint64_t seed, int32_t n, int32_t nx_min, int32_t nx_max,
                               lulesh_instance* out);

int lulesh_ens_create(const lulesh_instance* instances, int32_t n, int32_t mode, int32_t device,
                      lulesh_ensemble** out);
int lulesh_ens_destroy(lulesh_ensemble* ens);

/* examples/benchmark.jl's loop for every instance at once: each instance
 * steps until its time reaches stoptime or its cycle reaches num_iters.
 * Returns the first non-zero instance status (others keep running). */
int lulesh_ens_run(lulesh_ensemble* ens, int64_t num_iters);

/* Returns every instance to its initial state (as created). */
int lulesh_ens_reset(lulesh_ensemble* ens);

int lulesh_ens_sizes(const lulesh_ensemble* ens, int32_t* n, int64_t* total_elem, int64_t* total_node);
int lulesh_ens_get_scalars(const lulesh_ensemble* ens, int32_t instance, lulesh_scalars* out);
int lulesh_ens_field_length(const lulesh_ensemble* ens, int32_t instance, int32_t field, int64_t* count);
/* FP64 element and node fields of one instance (index fields: use a single
 * problem handle). */
int lulesh_ens_download_field(lulesh_ensemble* ens, int32_t instance, int32_t field, void* host,
                              int64_t count);
int lulesh_ens_get_stream(lulesh_ensemble* ens, void** stream);
int lulesh_ens_get_tuning(const lulesh_ensemble* ens, lulesh_tuning* out);
int lulesh_ens_set_tuning(lulesh_ensemble* ens, const lulesh_tuning* t);
int lulesh_ens_autotune(lulesh_ensemble* ens, int32_t cycles, lulesh_tuning* chosen);

/* Splits instances over `parts` GPUs (one rank each) for a run with no
 * data-path collective: longest-processing-time greedy on the cost nx^3
 * (largest first, ties by index), each instance to the part with the least
 * cost so far (ties to the lowest part). part_of[i] receives instance i's
 * part. Host only; deterministic, so every rank computes the same split. */
int lulesh_ens_partition(const lulesh_instance* instances, int32_t n, int32_t parts, int32_t* part_of);

/* Diagnostic without a reference counterpart: measures the device's FP64
 * FMA and add issue rates (instructions per second), the roof this FP64
 * step is bound by. */
int lulesh_measure_fp64_peak(int32_t device, double* fma_per_s, double* add_per_s);

/* ---- Nodal forces without device allocation -----------------------------
 * No counterpart in the reference. For callers that keep the Domain's arrays
 * in device memory they manage themselves and must not let a library
 * allocate device memory (for example a Julia program whose CuArrays come
 * from its own memory pool, or an application that budgets every byte of
 * device memory up front). The caller passes device pointers to its own
 * arrays in the reference's Domain layout; the corner-force scratch the
 * computation needs is a fixed array inside the library, so the call makes no
 * cudaMalloc, cudaFree or other allocating call.
 *   - at most LULESH_STATIC_MAX_ELEMS elements; larger problems are rejected
 *     with LULESH_ERR_ARGUMENT.
 *   - the fixed array (6 MiB) is committed on a device by the first call
 *     there (CUDA loads the library's device code lazily), not when the
 *     library is loaded; it then stays until the process exits. On a device
 *     with no free memory that first call returns LULESH_ERR_CUDA.
 *   - every call shares that array: calls that overlap on the GPU (two
 *     streams or two host threads at once) race and give wrong forces.
 *   - the first call on a device looks up the array's address on that
 *     device; make it before any stream capture.
 * Computes the nodal forces fx, fy, fz (stress plus hourglass forces) of the
 * given state on `stream` (a cudaStream_t, 0 for the legacy default stream),
 * then copies a status word to the host and synchronizes that stream before
 * returning. The forces agree with those of the step's own force kernel to
 * 1e-8 relative, not bitwise: here each corner's stress and hourglass terms
 * are added before the node sum.
 * Returns LULESH_ERR_VOLUME with *site LULESH_SITE_EARLY (an element's
 * Jacobian determinant <= 0) or LULESH_SITE_HOURGLASS (a relative volume
 * <= 0). */
#define LULESH_STATIC_MAX_ELEMS 32768

typedef struct {
  int64_t num_elem, num_node;
  const int64_t* nodelist;            /* 8*num_elem, element-major, 0-based node ids */
  const int64_t* nodeElemStart;       /* num_node, 0-based offsets into nodeElemCornerList */
  const int64_t* nodeElemCount;       /* num_node */
  const int64_t* nodeElemCornerList;  /* 8*num_elem, 1-based corner ids 8*e + c + 1 */
  const double *x, *y, *z, *xd, *yd, *zd;          /* num_node */
  const double *p, *q, *ss, *v, *volo, *elemMass;  /* num_elem */
  double hgcoef;
  int32_t mode;                       /* LULESH_MODE_* bits */
  double *fx, *fy, *fz;               /* num_node outputs */
} lulesh_force_args;

int lulesh_calc_force_for_nodes_static(const lulesh_force_args* args, void* stream, int32_t* site);

/* ---- Reverse-mode adjoint of a run -------------------------------------------
 * The reference differentiates its step with Enzyme (the optional Enzyme
 * extension of LULESH.jl); this is a hand-written adjoint of the same run.
 * The objective of the state S after the run is
 *     L(S) = sum_e w_e e_e + sum_n 0.5 w_n |u_n|^2,
 * w_e = elemMass_e if the element's centroid in the initial mesh lies
 * within `radius` of the origin (else 0), w_n = nodalMass_n likewise for the
 * node's initial position: the total energy within that radius. Callers can
 * replace it with a linear objective sum_f <seed_f, field_f> over state fields
 * (lulesh_adj_set_seed). The state fields are x y z xd yd zd (node) and e p q
 * v ss (element); the gradient w.r.t. the run's initial value of each is
 * returned (lulesh_adj_get_gradient), with dL/dhgcoef in the result.
 * Memory: one state per checkpoint plus checkpoint_every cycles of tape
 * (about 8*(204*E + 6*N) bytes per taped cycle); a second tape of the same
 * size, allocated at the first gradient that has two or more segments if it
 * fits, lets the recompute of one segment overlap the transpose of the next
 * freely; without it they overlap on one tape (lulesh_adj_set_overlap). The derivative is that of the branches the
 * forward run took (dt minima, clamps, limiter cases). */
typedef struct lulesh_adjoint lulesh_adjoint;

typedef struct {
  double loss;          /* L at the end of the run */
  double grad_hgcoef;   /* dL/dhgcoef */
  double forward_ms;    /* checkpointed forward sweep, host wall clock */
  double reverse_ms;    /* objective + recompute + transpose, host wall clock */
  int64_t cycles;
  int32_t checkpoints;
  int32_t status;
  int32_t sweep;        /* reverse sweep taken: 0 sequential, 1 overlapped on two tapes, 2 on one */
  int32_t reserved;
} lulesh_adj_result;

int lulesh_adj_create(lulesh_domain* dom, double radius, int32_t checkpoint_every, lulesh_adjoint** out);
int lulesh_adj_destroy(lulesh_adjoint* adj);
/* Linear objective weights for one state field (replaces the energy
 * objective until lulesh_adj_clear_seeds). */
int lulesh_adj_set_seed(lulesh_adjoint* adj, int32_t field, const double* weights, int64_t count);
int lulesh_adj_clear_seeds(lulesh_adjoint* adj);
/* The objective at the domain's current state. */
int lulesh_adj_loss(lulesh_adjoint* adj, double* loss);
/* Runs up to num_cycles cycles (timeIncrement! + lagrangeLeapFrog each; fewer
 * if time reaches stoptime first) from the domain's current state, leaves the
 * domain at the final state, and computes the gradient of the objective
 * w.r.t. the initial state and hgcoef. result->cycles is the number run. */
int lulesh_adj_gradient(lulesh_adjoint* adj, int64_t num_cycles, lulesh_adj_result* result);
int lulesh_adj_get_gradient(lulesh_adjoint* adj, int32_t field, double* host, int64_t count);
/* mode = 0: one tape, each segment recomputed and then transposed on the
 * domain's stream. mode = 1 (the default): each segment's recompute overlaps
 * the transpose of the next, on two tapes where the second fits (allocated
 * by the first gradient with two or more segments), else on one tape (the
 * recompute fills each tape slot once the transpose has released it).
 * mode = 2: overlapped on one tape. Modes 0 and 2 free the second tape. The
 * plan a gradient took is in lulesh_adj_result.sweep; gradients are bitwise
 * the same for every mode. */
int lulesh_adj_set_overlap(lulesh_adjoint* adj, int32_t mode);

/* Human-readable text of a status code. */
const char* lulesh_status_string(int32_t status);

#ifdef __cplusplus
}
#endif

#endif /* LULESH_GB300_H */
