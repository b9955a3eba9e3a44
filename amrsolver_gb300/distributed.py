"""A level of boxes sharded over the ranks of a torch.distributed group.

The reference runs a level as a MultiFab whose boxes are spread over MPI
ranks: every stage's FillPatch exchanges the 3-cell halo between ranks
(src/tim/CNS_advance.cpp:50-56 and the later stage calls) and the time step
is a ReduceRealMin over ranks (src/CNS.cpp:392).  Here one process drives one
GPU:

* `partition` assigns the boxes to ranks by cost (cells of the grown box, the
  work a stage does for it), largest first onto the least-loaded rank.
* `HaloPlan` maps every ghost cell of every box to the domain cell it copies
  (periodic wrap, foextrap clamp, reflection with the sign flips of the BC
  table; the mapping of the library's own level fill) and to the box owning
  that cell.  Every rank builds the same plan for the whole level, so the
  sender of a halo slab knows, without asking, which cells the receiver
  wants and in which order.
* `DistributedLevel.fill` packs the requested cells of each local box into
  one buffer per destination rank, exchanges the buffers with
  torch.distributed point-to-point calls (NCCL between GPUs, gloo on CPU) and
  scatters them into the ghost cells, sign included.  Copies land in each
  rank's own buffers; no kernel reads another GPU's memory.  Cells whose
  source is local take the same path without the exchange.
* `DistributedLevel.est_time_step` is the local cns_estdt minimum followed
  by an all-reduce(MIN).

The stage arithmetic is the library's: the local boxes form one box list
(ghosts left as the fill wrote them) and each stage is amrs_rk_stage_boxlist.
Ghost cells beyond ext_dir sides (codes 1 and 6) are the problem's bcnormal's
and are not filled here.
"""
from __future__ import annotations

import numpy as np
import torch

from .problems import NCONS, NGHOST

G = NGHOST


def partition(costs, nranks):
    """Rank of every box: largest cost first onto the least-loaded rank (ties
    to the lower rank; boxes of equal cost in index order)."""
    load = [0.0] * nranks
    rank = [0] * len(costs)
    for b in sorted(range(len(costs)), key=lambda b: (-costs[b], b)):
        r = min(range(nranks), key=lambda q: (load[q], q))
        rank[b] = r
        load[r] += costs[b]
    return rank


def grown_cells(n):
    return (n[0] + 2 * G) * (n[1] + 2 * G) * (n[2] + 2 * G)


def _map_axis(c, d, lo, hi, bcl, bch):
    """Source coordinate along axis d and, per component, whether that axis
    flips the sign (reflect_odd), for coordinates `c` (numpy ints).
    Returns (src, flip[NCONS, len(c)], ext) where ext marks coordinates
    beyond an ext_dir side (codes 1, 6)."""
    n = hi - lo + 1
    src = c.copy()
    flip = np.zeros((NCONS,) + c.shape, dtype=bool)
    ext = np.zeros(c.shape, dtype=bool)
    for side, phys in ((0, bcl), (1, bch)):
        m = (c < lo) if side == 0 else (c > hi)
        if not m.any():
            continue
        if phys in (1, 6):
            ext |= m
            continue
        if phys == -1:
            src[m] = lo + np.mod(c[m] - lo, n)
        elif phys == 2:
            src[m] = lo if side == 0 else hi
        elif phys in (3, 4, 5):
            src[m] = (2 * lo - c[m] - 1) if side == 0 else (2 * hi - c[m] + 1)
        else:
            raise ValueError("unsupported boundary code %d" % phys)
        if phys in (3, 4, 5):
            for comp in range(NCONS):
                vel = 1 <= comp <= 3
                normal = comp == 1 + d
                odd = (vel and normal) if phys in (3, 4) else vel
                if odd:
                    flip[comp][m] = True
    return src, flip, ext


class HaloPlan:
    """Ghost-cell sources of a level of boxes tiling a domain.

    boxes: list of (lo, n) with n = (nx, ny, nz); domain: (lo, n); bc_lo /
    bc_hi: cns.lo_bc / cns.hi_bc codes per direction.  For box b the plan
    holds, over the ghost cells of grow(b, 3) that are filled (not beyond an
    ext_dir side), flat offsets into b's ghosted array (`ghost`), the owning
    box of the source cell (`src_box`), the flat offset of the source cell in
    that box's ghosted array (`src_off`) and a sign per component
    (`sign`, NCONS x cells: -1 where an odd reflection flips it)."""

    def __init__(self, boxes, domain, bc_lo, bc_hi):
        self.boxes = [(tuple(int(v) for v in lo), tuple(int(v) for v in n)) for lo, n in boxes]
        dlo, dn = (tuple(int(v) for v in domain[0]), tuple(int(v) for v in domain[1]))
        self.domain = (dlo, dn)
        dhi = tuple(dlo[d] + dn[d] - 1 for d in range(3))
        for d in range(3):
            if (bc_lo[d] == -1) != (bc_hi[d] == -1):
                raise ValueError("periodic on one side only in direction %d" % d)
        # owner of every domain cell (z, y, x order)
        owner = np.full((dn[2], dn[1], dn[0]), -1, dtype=np.int32)
        for b, (lo, n) in enumerate(self.boxes):
            sl = tuple(slice(lo[d] - dlo[d], lo[d] - dlo[d] + n[d]) for d in (2, 1, 0))
            if any(s.start < 0 or s.stop > dn[d] for s, d in zip(sl, (2, 1, 0))):
                raise ValueError("box %d lies outside the domain" % b)
            if (owner[sl] != -1).any():
                raise ValueError("box %d overlaps another box" % b)
            owner[sl] = b
        if (owner < 0).any():
            raise ValueError("the boxes do not cover the domain")
        self.ghost, self.src_box, self.src_off, self.sign = [], [], [], []
        for b, (lo, n) in enumerate(self.boxes):
            gx = np.arange(lo[0] - G, lo[0] + n[0] + G)
            gy = np.arange(lo[1] - G, lo[1] + n[1] + G)
            gz = np.arange(lo[2] - G, lo[2] + n[2] + G)
            K, J, I = np.meshgrid(gz, gy, gx, indexing="ij")
            inside = ((I >= lo[0]) & (I < lo[0] + n[0]) & (J >= lo[1]) & (J < lo[1] + n[1]) & (K >= lo[2])
                      & (K < lo[2] + n[2]))
            flat = np.nonzero(~inside.ravel())[0]
            ci, cj, ck = I.ravel()[flat], J.ravel()[flat], K.ravel()[flat]
            srcs, flips, exts = [], [], []
            for d, c in enumerate((ci, cj, ck)):
                s, f, e = _map_axis(c, d, dlo[d], dhi[d], bc_lo[d], bc_hi[d])
                srcs.append(s)
                flips.append(f)
                exts.append(e)
            keep = ~(exts[0] | exts[1] | exts[2])
            si, sj, sk = (s[keep] for s in srcs)
            flip = (flips[0] ^ flips[1] ^ flips[2])[:, keep]
            ob = owner[sk - dlo[2], sj - dlo[1], si - dlo[0]]
            # source offsets in the owners' ghosted arrays
            olo = np.array([self.boxes[q][0] for q in range(len(self.boxes))])[ob]
            on = np.array([self.boxes[q][1] for q in range(len(self.boxes))])[ob]
            nxg, nyg = on[:, 0] + 2 * G, on[:, 1] + 2 * G
            off = ((sk - olo[:, 2] + G) * nyg + (sj - olo[:, 1] + G)) * nxg + (si - olo[:, 0] + G)
            self.ghost.append(flat[keep].astype(np.int64))
            self.src_box.append(ob.astype(np.int64))
            self.src_off.append(off.astype(np.int64))
            self.sign.append(np.where(flip, -1.0, 1.0))


class DistributedLevel:
    """A level sharded over the ranks of `group` (the default group when
    None); each rank holds the boxes `partition` gives it, three ghosted
    state slots each, on `device`.

    boxes: list of (lo, n); fields: the ghosted initial field of every box
    (numpy arrays, callables returning one, or None for the boxes of other
    ranks); backend: a callable that takes the level and returns the object
    running its stages and local dt; by default `LibraryBackend`, the
    library's box list on this rank's GPU."""

    def __init__(self, scheme, closures, boxes, fields, dx, domain, bc_lo, bc_hi, group=None, device=None,
                 backend=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group) if dist.is_initialized() else 0
        self.world = dist.get_world_size(group) if dist.is_initialized() else 1
        self.scheme, self.closures = scheme, closures
        self.dx = tuple(float(v) for v in dx)
        self.bc_lo, self.bc_hi = tuple(bc_lo), tuple(bc_hi)
        self.boxes = [(tuple(lo), tuple(n)) for lo, n in boxes]
        self.box_rank = partition([grown_cells(n) for _, n in self.boxes], self.world)
        self.local = [b for b in range(len(self.boxes)) if self.box_rank[b] == self.rank]
        self.lidx = {b: i for i, b in enumerate(self.local)}
        self.device = torch.device(device) if device is not None else torch.device("cpu")
        self.plan = HaloPlan(self.boxes, domain, bc_lo, bc_hi)
        self.slots = []
        for b in self.local:
            f = fields[b]() if callable(fields[b]) else fields[b]
            t = torch.as_tensor(np.ascontiguousarray(f, dtype=np.float64)).to(self.device)
            self.slots.append([t, t.clone(), t.clone()])
        self._build_exchange()
        self.backend = (backend or LibraryBackend)(self)
        self.cur = 0
        self.time = 0.0

    # ---------------------------------------------------------- plan --
    def _build_exchange(self):
        """Per destination rank: the local source cells to pack, grouped by
        source box; per source rank: where the received cells go, grouped by
        destination box.  Entries are ordered by (destination box, ghost
        cell), which both sides derive from the same global plan."""
        P, dev = self.plan, self.device
        me = self.rank
        rank_of = np.array(self.box_rank)
        self.send = {}   # dst rank -> (count, [(local src box, src_off, pos)])
        self.recv = {}   # src rank -> (count, [(local dst box, ghost, pos, sign)])
        for d in range(self.world):
            pos0 = 0
            groups = {}
            for b in range(len(self.boxes)):
                if self.box_rank[b] != d:
                    continue
                sel = np.nonzero(rank_of[P.src_box[b]] == me)[0]
                if sel.size == 0:
                    continue
                qs = P.src_box[b][sel]
                pos = pos0 + np.arange(sel.size)
                for q in np.unique(qs):
                    m = qs == q
                    groups.setdefault(int(q), ([], []))
                    groups[int(q)][0].append(P.src_off[b][sel][m])
                    groups[int(q)][1].append(pos[m])
                pos0 += sel.size
            if pos0:
                self.send[d] = (pos0, [(self.lidx[q], torch.as_tensor(np.concatenate(o), device=dev),
                                        torch.as_tensor(np.concatenate(p), device=dev))
                                       for q, (o, p) in sorted(groups.items())])
        for s in range(self.world):
            pos0 = 0
            items = []
            for b in self.local:
                sel = np.nonzero(rank_of[P.src_box[b]] == s)[0]
                if sel.size == 0:
                    continue
                items.append((self.lidx[b], torch.as_tensor(P.ghost[b][sel], device=dev),
                              torch.as_tensor(pos0 + np.arange(sel.size), device=dev),
                              torch.as_tensor(np.ascontiguousarray(P.sign[b][:, sel]), device=dev)))
                pos0 += sel.size
            if pos0:
                self.recv[s] = (pos0, items)

    # ---------------------------------------------------------- halo --
    def fill(self, slot):
        """FillPatch of state slot `slot` across the whole level."""
        bufs = {}
        for d, (count, groups) in self.send.items():
            buf = torch.empty((NCONS, count), dtype=torch.float64, device=self.device)
            for q, off, pos in groups:
                buf[:, pos] = self.slots[q][slot].view(NCONS, -1)[:, off]
            bufs[d] = buf
        rbufs = {}
        ops = []
        for s, (count, _) in self.recv.items():
            if s == self.rank:
                rbufs[s] = bufs[s]
            else:
                rbufs[s] = torch.empty((NCONS, count), dtype=torch.float64, device=self.device)
                ops.append(self.dist.P2POp(self.dist.irecv, rbufs[s], s, self.group))
        for d, buf in bufs.items():
            if d != self.rank:
                ops.append(self.dist.P2POp(self.dist.isend, buf, d, self.group))
        if ops:
            for r in self.dist.batch_isend_irecv(ops):
                r.wait()
        for s, (_, items) in self.recv.items():
            rb = rbufs[s]
            for b, ghost, pos, sign in items:
                self.slots[b][slot].view(NCONS, -1)[:, ghost] = rb[:, pos] * sign

    # ---------------------------------------------------------- steps --
    def advance(self, dt, order_rk=3, stages_rk=3):
        """One CNS::advance step of the level (src/tim/CNS_advance.cpp:14-183):
        per stage the halo fill across ranks, then the stage on every local
        box."""
        from . import capi
        progs = capi.rk_program(order_rk, stages_rk, dt)
        s1 = self.cur
        work = [i for i in range(3) if i != s1]
        cur, which = s1, 0
        for p in progs:
            src = s1 if p.src_state == 0 else cur
            out = work[which]
            if out == src:
                which ^= 1
                out = work[which]
            self.fill(src)
            self.backend.stage(p, src, s1, out)
            cur = out
            which ^= 1
        self.cur = cur
        self.time += dt
        return dt

    def est_time_step(self, cfl):
        """CNS::estTimeStep over the level: the local minimum of cns_estdt,
        then an all-reduce(MIN) over the ranks (src/CNS.cpp:380-395)."""
        t = torch.tensor([self.backend.local_dt(cfl, self.cur)], dtype=torch.float64,
                         device=self.backend.reduce_device)
        if self.world > 1:
            self.dist.all_reduce(t, op=self.dist.ReduceOp.MIN, group=self.group)
        return float(t.item())

    def valid(self, b):
        """Valid cells of local box b (global index) in the current slot."""
        return self.slots[self.lidx[b]][self.cur][:, G:-G, G:-G, G:-G]

    def close(self):
        """Release the backend's library objects (box list before handle)."""
        close = getattr(self.backend, "close", None)
        if close:
            close()


class LibraryBackend:
    """Stages of the local boxes through the library: one box list of the
    rank's boxes (no ghost fill of its own: the level's fill wrote the
    ghosts), one amrs_rk_stage_boxlist per stage."""

    def __init__(self, lev):
        from . import capi
        dev = lev.device
        if dev.type != "cuda":
            raise RuntimeError("the library backend needs the rank's CUDA device")
        self.h = capi.Handle(lev.scheme, lev.closures, dev.index or 0)
        # what the dt reduction reads, not the level itself (no reference cycle)
        self.slots, self.dx = lev.slots, lev.dx
        self.los = [lev.boxes[b][0] for b in lev.local]
        self.bl = capi.BoxList(self.h, self.los, lev.slots, [1.0 / v for v in lev.dx]) if lev.local else None
        self.reduce_device = dev
        self._dt = torch.empty(1, dtype=torch.float64, device=dev)

    def close(self):
        if self.bl is not None:
            self.bl.close()
            self.bl = None
        self.h.close()

    def stage(self, prog, s_in, s1, s_out):
        if self.bl is not None:
            self.bl.stage(prog, s_in, s1, s_out)

    def local_dt(self, cfl, slot):
        best = float("inf")
        for i, lo in enumerate(self.los):
            self.h.est_timestep(self.slots[i][slot], self.dx, cfl, self._dt, lo=lo)
            best = min(best, float(self._dt.item()))
        return best
