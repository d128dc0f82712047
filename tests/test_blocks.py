"""The multi-rank decomposition on CPU: the tp^3 block plan of the
(tp*nx)^3 mesh (initMeshDecomp, src/LULESH.jl:62-97) and its halo plan,
computed by the library on the host (lulesh_block_plan, no GPU), and the halo
exchange run as it would between GPUs, over gloo ranks that each own some of
the blocks (world sizes 2 and 8)."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def coords(ids, edge):
    """(i, j, k) of x-fastest ids in a cube of `edge` per side."""
    ids = np.asarray(ids, dtype=np.int64)
    return ids % edge, (ids // edge) % edge, ids // (edge * edge)


@pytest.mark.parametrize("nx,tp,mode", [(3, 2, 0), (3, 2, 7), (2, 3, 0), (4, 3, 4)])
def test_block_plan_partitions_the_mesh(gpu_lib, nx, tp, mode):
    p = gpu_lib.block_plan(nx, tp, mode)
    nxg, nb = nx * tp, tp ** 3
    Eb, Nb = nx ** 3, (nx + 1) ** 3
    assert p["E"] == nb * Eb and p["N"] == nb * Nb
    # every element once, in blocks of the reference's rank order
    assert np.array_equal(np.sort(p["elem_global"]), np.arange(nxg ** 3))
    assert set(p["node_global"].tolist()) == set(range((nxg + 1) ** 3))
    for b in range(nb):
        col, row, plane = b % tp, (b // tp) % tp, b // (tp * tp)
        i, j, k = coords(p["elem_global"][b * Eb:(b + 1) * Eb], nxg)
        assert i.min() == col * nx and i.max() == col * nx + nx - 1
        assert j.min() == row * nx and k.min() == plane * nx
        # per-rank order: x fastest, then y, then z
        assert np.all(np.diff(p["elem_global"][b * Eb:(b + 1) * Eb]) > 0)
        i, j, k = coords(p["node_global"][b * Nb:(b + 1) * Nb], nxg + 1)
        assert i.min() == col * nx and i.max() == col * nx + nx
        assert k.min() == plane * nx and k.max() == plane * nx + nx


@pytest.mark.parametrize("nx,tp,mode", [(3, 2, 0), (3, 2, 7), (2, 3, 0)])
def test_halo_sources_cross_a_block_face(gpu_lib, nx, tp, mode):
    p = gpu_lib.block_plan(nx, tp, mode)
    nxg, E, Eb = nx * tp, p["E"], nx ** 3
    # a ghost delv slot copies an element of another block beside the slot's block
    src_blk = p["halo_delv_src"] // Eb
    assert np.all(src_blk != p["halo_delv_dst"])
    si, sj, sk = coords(p["elem_global"][p["halo_delv_src"]], nxg)
    d = p["halo_delv_dst"]
    lo = lambda c: c * nx
    di = np.maximum(0, np.maximum(lo(d % tp) - si, si - (lo(d % tp) + nx - 1)))
    dj = np.maximum(0, np.maximum(lo((d // tp) % tp) - sj, sj - (lo((d // tp) % tp) + nx - 1)))
    dk = np.maximum(0, np.maximum(lo(d // (tp * tp)) - sk, sk - (lo(d // (tp * tp)) + nx - 1)))
    assert np.all(di + dj + dk == 1)
    # the faithful xi-plus read is the element itself: no ghost in +x
    if not mode & 4:
        assert not np.any(si > lo(d % tp) + nx - 1)
    # a ghost corner copies a corner of another block's element whose node the slot's block holds
    c, pe = p["halo_corner_src"] // E, p["halo_corner_src"] % E
    assert np.all(pe // Eb != p["halo_corner_dst"])
    gi, gj, gk = coords(p["elem_global"][pe], nxg)
    # the corner's node: +1 in x for corners 1, 2, 5, 6; in y for 2, 3, 6, 7; in z for 4..7
    ni = gi + np.isin(c, [1, 2, 5, 6]); nj = gj + np.isin(c, [2, 3, 6, 7]); nk = gk + (c >= 4)
    d = p["halo_corner_dst"]
    for n_, off in ((ni, d % tp), (nj, (d // tp) % tp), (nk, d // (tp * tp))):
        assert np.all((n_ >= off * nx) & (n_ <= off * nx + nx))
    # every slot once per (block, source)
    assert len(set(zip(p["halo_corner_dst"].tolist(), p["halo_corner_src"].tolist()))) == c.size


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _exchange(values, src, dst_blk, src_blk, owner, rank, world):
    """Fills the ghost slots this rank holds (dst block owned here) with the
    values their sources hold: a local copy, or point-to-point messages with
    every other rank, both sides walking the plan in slot order."""
    got = np.full(src.size, np.nan)
    mine = owner[dst_blk] == rank
    local = mine & (owner[src_blk] == rank)
    got[local] = values[src[local]]
    reqs, bufs = [], {}
    for peer in range(world):
        if peer == rank:
            continue
        send = (owner[dst_blk] == peer) & (owner[src_blk] == rank)
        recv = mine & (owner[src_blk] == peer)
        if send.any():
            reqs.append(dist.isend(torch.from_numpy(values[src[send]].copy()), dst=peer))
        if recv.any():
            bufs[peer] = (recv, torch.empty(int(recv.sum()), dtype=torch.float64))
            reqs.append(dist.irecv(bufs[peer][1], src=peer))
    for r in reqs:
        r.wait()
    for peer, (recv, buf) in bufs.items():
        got[recv] = buf.numpy()
    return got, mine


def _worker(rank, world, port, nx, tp, q):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "lulesh.jl_gb300"))
    import lulesh_gb300 as L
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        p = L.block_plan(nx, tp, 7)
        E, Eb, nb = p["E"], nx ** 3, tp ** 3
        owner = np.arange(nb) % world  # block b lives on rank b % world
        Eglob = (nx * tp) ** 3
        # stand-ins for the exchanged values that name where they came from:
        # an element's whole-mesh id (delv), a corner's whole-mesh corner id
        delv = p["elem_global"].astype(np.float64)
        c = np.arange(8 * E) // E
        corner = (c * Eglob + p["elem_global"][np.arange(8 * E) % E]).astype(np.float64)
        gd, mine_d = _exchange(delv, p["halo_delv_src"], p["halo_delv_dst"], p["halo_delv_src"] // Eb,
                               owner, rank, world)
        gc, mine_c = _exchange(corner, p["halo_corner_src"], p["halo_corner_dst"],
                               (p["halo_corner_src"] % E) // Eb, owner, rank, world)
        ok_d = np.array_equal(gd[mine_d], delv[p["halo_delv_src"][mine_d]])
        ok_c = np.array_equal(gc[mine_c], corner[p["halo_corner_src"][mine_c]])
        counts = [None] * world
        dist.all_gather_object(counts, (int(mine_d.sum()), int(mine_c.sum()), ok_d, ok_c))
        if rank == 0:
            q.put((counts, int(p["halo_delv_src"].size), int(p["halo_corner_src"].size)))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(300)
@pytest.mark.parametrize("world", [2, 8])
def test_halo_exchange_over_gloo_ranks(gpu_lib, world):
    nx, tp = 3, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, nx, tp, q)) for r in range(world)]
    for p in procs:
        p.start()
    counts, nd, nc = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(ok_d and ok_c for _, _, ok_d, ok_c in counts)
    assert sum(d for d, _, _, _ in counts) == nd and sum(c for _, c, _, _ in counts) == nc


def test_block_plan_edges_and_limits(gpu_lib):
    import ctypes
    L = gpu_lib.load_library()
    # one block: the whole mesh, no ghost slots
    p = gpu_lib.block_plan(4, 1, 0)
    assert p["E"] == 64 and p["N"] == 125
    assert p["halo_delv_src"].size == 0 and p["halo_corner_src"].size == 0
    assert np.array_equal(p["elem_global"], np.arange(64)) and np.array_equal(p["node_global"], np.arange(125))
    assert p["corner_list_entries"] == 8 * 64
    # rejected before any work: empty blocks, a bad mode, a mesh past the index limit
    sizes = (ctypes.c_int64 * 5)()
    assert L.lulesh_block_plan_sizes(0, 2, 0, sizes) == 6
    assert L.lulesh_block_plan_sizes(3, 0, 0, sizes) == 6
    assert L.lulesh_block_plan_sizes(3, 2, 9, sizes) == 6
    assert L.lulesh_block_plan_sizes(301, 2, 0, sizes) == 6
