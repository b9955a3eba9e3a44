"""A level sharded over two ranks (gloo, CPU): cost partition, halo exchange
between the ranks' own buffers, dt all-reduce(MIN).

The stages run through a test backend that applies the CPU oracle box by
box (the library's kernels need a GPU); what is under test is the
distributed layer: every ghost cell after the exchange must equal the fill
of one box covering the domain, two SSPRK3 steps of the sharded level must
equal the oracle's single-box run bit for bit, and the all-reduced dt must
equal the single-box estimate.  Reference: src/tim/CNS_advance.cpp:50-56
(FillPatch at every stage), src/CNS.cpp:392 (ReduceRealMin of the dt).
"""
import os
import socket

import numpy as np
import pytest

from amrsolver_gb300 import problems as P

G = P.NGHOST

CASES = {
    # periodic TGV split into uneven boxes
    "periodic": dict(n=(16, 12, 10), cuts=([5, 11], [7], [4]), bc_lo=(-1, -1, -1), bc_hi=(-1, -1, -1)),
    # x periodic, y outflow / symmetry, z slip wall / no-slip wall
    "walls": dict(n=(14, 12, 9), cuts=([6], [3, 8], [5]), bc_lo=(-1, 2, 4), bc_hi=(-1, 3, 5)),
}


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _domain_field(case):
    n = CASES[case]["n"]
    if case == "periodic":
        U, dx = P.tgv(16, mach=0.2)
        U = U[:, :n[2] + 2 * G, :n[1] + 2 * G, :n[0] + 2 * G].copy()
        return U, dx
    return P.random_state(n, seed=5, amp=0.2), (0.11, 0.13, 0.17)


def _boxes(case):
    c = CASES[case]
    n = c["n"]
    edges = [[0] + list(cu) + [n[d]] for d, cu in enumerate(c["cuts"])]
    out = []
    for z0, z1 in zip(edges[2][:-1], edges[2][1:]):
        for y0, y1 in zip(edges[1][:-1], edges[1][1:]):
            for x0, x1 in zip(edges[0][:-1], edges[0][1:]):
                out.append(((x0, y0, z0), (x1 - x0, y1 - y0, z1 - z0)))
    return out


def _cut(U, lo, n):
    """Box (lo, n) of a ghosted domain field, ghosts included."""
    x0, y0, z0 = lo
    return U[:, z0:z0 + n[2] + 2 * G, y0:y0 + n[1] + 2 * G, x0:x0 + n[0] + 2 * G].copy()


class OracleBackend:
    """Stages of the local boxes with the CPU oracle (test only)."""

    def __init__(self, lev, orc):
        self.lev, self.orc = lev, orc
        self.reduce_device = "cpu"

    def stage(self, prog, s_in, s1, s_out):
        lev = self.lev
        dxinv = [1.0 / v for v in lev.dx]
        v = (slice(None), slice(G, -G), slice(G, -G), slice(G, -G))
        for i, b in enumerate(lev.local):
            lo = lev.boxes[b][0]
            S = lev.slots[i]
            Uin = S[s_in].numpy()
            reg = [S[s1].numpy()[v].copy(), Uin[v].copy(), self.orc.rhs(lev.scheme, lev.closures, Uin, dxinv, lo=lo)]
            for o in range(prog.nops):
                q = prog.ops[o]
                if q.kind == 0:
                    reg[q.dst] = q.a * reg[q.x] + q.b * reg[q.y]
                elif q.kind == 1:
                    reg[q.dst] = reg[q.dst] + q.a * reg[q.x]
                elif q.kind == 2:
                    reg[q.dst] = reg[q.x] + q.a * reg[q.dst]
                else:
                    reg[q.dst] = reg[q.x].copy()
            S[s_out].numpy()[v] = reg[1]

    def local_dt(self, cfl, slot):
        lev = self.lev
        return min(self.orc.est_timestep(lev.closures, lev.slots[i][slot].numpy(), lev.dx, cfl, lo=lev.boxes[b][0])
                   for i, b in enumerate(lev.local))


def _worker(rank, world, port, case, errfile):
    import torch
    import torch.distributed as dist

    from amrsolver_gb300 import distributed as D
    from oracle import pyoracle
    try:
        os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        dist.init_process_group("gloo", rank=rank, world_size=world)
        orc = pyoracle.oracle()
        c = CASES[case]
        U, dx = _domain_field(case)
        boxes = _boxes(case)
        fields = [(lambda lo=lo, n=n: _cut(U, lo, n)) for lo, n in boxes]
        sc = P.Scheme(flux_euler=1, order_keep=4, rhs_visc=1)
        cl = P.Closures.nondimensional(1.0 / 500.0)
        lev = D.DistributedLevel(sc, cl, boxes, fields, dx, ((0, 0, 0), c["n"]), c["bc_lo"], c["bc_hi"],
                                 backend=lambda lv: OracleBackend(lv, orc))
        assert sorted(set(lev.box_rank)) == list(range(world)) and len(lev.local) >= 1
        # halo exchange: every local box equals the single-box fill of the domain, ghosts included
        Uf = U.copy()
        orc.fill_halo(Uf, c["bc_lo"], c["bc_hi"])
        for i, b in enumerate(lev.local):
            lev.slots[i][0].fill_(float("nan"))  # ghosts: only the exchange may write them
            lev.slots[i][0][:, G:-G, G:-G, G:-G] = torch.from_numpy(_cut(U, *boxes[b])[:, G:-G, G:-G, G:-G])
        lev.fill(0)
        for i, b in enumerate(lev.local):
            np.testing.assert_array_equal(lev.slots[i][0].numpy(), _cut(Uf, *boxes[b]))
        # dt: local minimum, all-reduce(MIN)
        dt = lev.est_time_step(0.3)
        assert dt == orc.est_timestep(cl, Uf, dx, 0.3)
        # two SSPRK3 steps of the sharded level against one box covering the domain
        S = Uf
        dxinv = [1.0 / v for v in dx]
        for _ in range(2):
            lev.advance(dt)
            S = orc.advance(sc, cl, S, dxinv, c["bc_lo"], c["bc_hi"], dt)
        for b in lev.local:
            lo, n = boxes[b]
            ref = S[:, G + lo[2]:G + lo[2] + n[2], G + lo[1]:G + lo[1] + n[1], G + lo[0]:G + lo[0] + n[0]]
            np.testing.assert_array_equal(lev.valid(b).numpy(), ref)
        dist.barrier()
        dist.destroy_process_group()
    except BaseException as e:  # report to the parent through a file
        with open(errfile, "a") as f:
            f.write("rank %d: %r\n" % (rank, e))
        raise


@pytest.mark.parametrize("case", sorted(CASES))
def test_two_rank_level_matches_single_box(case, tmp_path):
    import torch.multiprocessing as mp
    err = str(tmp_path / "err.txt")
    mp.start_processes(_worker, args=(2, _free_port(), case, err), nprocs=2, join=True, start_method="spawn")
    assert not os.path.exists(err), open(err).read()


def test_partition_balances_cost():
    from amrsolver_gb300 import distributed as D
    specs, _, _ = P.batched_boxes(nboxes=64, seed=3)
    costs = [D.grown_cells(s.shape) for s in specs]
    for nr in (2, 3, 4, 8):
        r = D.partition(costs, nr)
        loads = [sum(c for c, q in zip(costs, r) if q == k) for k in range(nr)]
        # LPT: no rank exceeds the mean by more than the largest box
        assert max(loads) <= sum(costs) / nr + max(costs)
        assert r == D.partition(costs, nr)  # deterministic


def test_halo_plan_rejects_bad_tilings():
    from amrsolver_gb300 import distributed as D
    with pytest.raises(ValueError):
        D.HaloPlan([((0, 0, 0), (4, 4, 4))], ((0, 0, 0), (4, 4, 5)), (-1,) * 3, (-1,) * 3)  # uncovered
    with pytest.raises(ValueError):
        D.HaloPlan([((0, 0, 0), (4, 4, 4)), ((2, 0, 0), (2, 4, 4))], ((0, 0, 0), (4, 4, 4)), (-1,) * 3, (-1,) * 3)
