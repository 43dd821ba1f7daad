"""The slab decomposition's protocol across processes, on CPU ranks over gloo.

The library's eu_domain_* runs its slabs on one device; across GPUs each
rank would own one slab and the same three exchanges would cross ranks:
  * the dt: every rank proposes cfl min(dx, dy) / (its maximum signal
    speed) and all take the smallest (an all-reduce MIN, which equals the
    undivided grid's dt bit for bit because x -> c / x is monotone and
    correctly rounded; src/cpu/solver_mpi.cpp:416-443 reduces the speed);
  * after the x-sweep, the two boundary rows of each slab's x-sweep output
    go to the neighbour's halo rows (src/cpu/solver_mpi.cpp:340-402,
    547-573), point-to-point;
  * the y-sweep then needs nothing else.
Here each world-size-2 gloo rank steps its slab with the CPU oracle's two
sweep halves (ghost sides between slabs of kind "halo", left to the
exchange), using the library's own partition (eu_domain_plan, callable
without a GPU), and the gathered grid must equal the undivided oracle run
bit for bit, for transmissive and reflective outer walls.
"""
import os
import socket

import numpy as np
import pytest

WORLD = 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, case, nsteps, outdir):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    import large_sys_eq_opt_gb300.euler2d as E
    P = O.Oracle("port")
    P.set_threads(2)
    nx, ny, ext, bc, solver = case
    G = O.Grid(nx, ny, *ext, bc=bc)
    U = P.init_shock_bubble(G) if bc[2] == "reflective" else P.init_blast(G)
    row0 = E.domain_plan(ny, world)
    j0, j1 = row0[rank], row0[rank + 1]
    dy = (ext[3] - ext[2]) / ny
    lbc = list(bc)
    if rank > 0:
        lbc[2] = "halo"
    if rank + 1 < world:
        lbc[3] = "halo"
    g = O.Grid(nx, j1 - j0, ext[0], ext[1], ext[2] + dy * j0, ext[2] + dy * j1, bc=tuple(lbc))
    assert (g.y_max - g.y_min) / g.ny == dy          # the slab's spacing is the grid's, bit for bit
    S = np.ascontiguousarray(U[j0:j1 + 4])           # own rows with their 2-row frame
    T = g.zeros()
    N = g.zeros()
    t = 0.0

    def exchange(A):
        """Halo rows of A (storage rows 0,1 and ny+2, ny+3) from the neighbours."""
        reqs = []
        m = g.ny
        if rank > 0:        # my first two interior rows go down, the lower rank's last two come up
            send = torch.from_numpy(np.ascontiguousarray(A[2:4]))
            recv = torch.empty_like(send)
            reqs += [dist.isend(send, rank - 1), dist.irecv(recv, rank - 1)]
        if rank + 1 < world:
            send_u = torch.from_numpy(np.ascontiguousarray(A[m:m + 2]))
            recv_u = torch.empty_like(send_u)
            reqs += [dist.isend(send_u, rank + 1), dist.irecv(recv_u, rank + 1)]
        for r in reqs:
            r.wait()
        if rank > 0:
            A[0:2] = recv.numpy()
        if rank + 1 < world:
            A[m + 2:m + 4] = recv_u.numpy()

    for _ in range(nsteps):
        P.apply_boundary(S, g)                       # outer sides only (halo sides untouched)
        d = torch.tensor([P.compute_dt(S, g, 0.8)], dtype=torch.float64)
        dist.all_reduce(d, op=dist.ReduceOp.MIN)
        dt = float(d.item())
        P.sweep_x(S, T, g, dt, solver)
        P.apply_boundary(T, g)
        exchange(T)
        P.sweep_y(T, N, g, dt, solver)
        P.apply_boundary(N, g)
        S, N = N, S
        t += dt
    np.save(os.path.join(outdir, f"slab{rank}.npy"), S[2:-2])
    np.save(os.path.join(outdir, f"t{rank}.npy"), np.array([t]))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("case", [
    (96, 64, (0.0, 2.0, 0.0, 2.0), ("transmissive",) * 4, "hllc"),
    (120, 50, (0.0, 0.225, 0.0, 0.089), ("transmissive", "transmissive", "reflective", "reflective"), "exact"),
])
def test_two_gloo_ranks_equal_the_undivided_grid(tmp_path, case):
    import torch.multiprocessing as mp
    from oracle import oracle as O
    O.build(reference=False)
    nsteps = 12
    port = _free_port()
    mp.start_processes(_rank_main, args=(WORLD, port, case, nsteps, str(tmp_path)), nprocs=WORLD,
                       start_method="spawn")
    P = O.Oracle("port")
    nx, ny, ext, bc, solver = case
    G = O.Grid(nx, ny, *ext, bc=bc)
    U = P.init_shock_bubble(G) if bc[2] == "reflective" else P.init_blast(G)
    ref = P.run(U, G, 0.8, 1e30, solver, max_steps=nsteps)
    got = np.concatenate([np.load(tmp_path / f"slab{r}.npy") for r in range(WORLD)])
    assert np.array_equal(got, U[2:-2]), float(np.abs(got - U[2:-2]).max())
    for r in range(WORLD):
        assert float(np.load(tmp_path / f"t{r}.npy")[0]) == ref["t"]
