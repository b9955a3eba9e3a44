"""AMReX plotfiles of a level, as the reference writes them for yt.

CNS::writePlotFile (src/CNS.cpp:644-874) writes, for each level, the
plotfile Header (the plotfile type, the variable names -- state components
first, then the derived quantities the run asked for, in the order they
were registered -- the dimension, time, finest level, problem extent,
refinement ratios, domain boxes, level steps, cell sizes, coordinate system,
boundary flag, then per level its boxes in physical coordinates and the path
of its MultiFab), and the level's data as one MultiFab through AMReX's
VisMF::Write.  The state components are density, xmom, ymom, zmom, energy
(src/set/CNS_setup.cpp:118-150); the derived ones pressure, temperature,
x_velocity, y_velocity, z_velocity (src/set/CNS_setup.cpp:153-176), computed
here on the device by amrs_plot_derive_box in the operation order of the
reference's derive functions.

The Header follows writePlotFile line by line (reals with 17 significant
digits, as AMReX's Amr sets its header stream).  The MultiFab is written in
the layout of AMReX's VisMF (version-1 header `Level_0/Cell_H` with the box
array, the offset of every FAB in the data file and per-FAB minima and
maxima; data file `Level_0/Cell_D_00000` with one FAB after another, each an
ASCII FAB header naming the IEEE little-endian double format and the box,
then the values, component by component, i fastest).  AMReX is not part of
the reference tree, so this layout is restated from AMReX's format and is
checked only by `read_plotfile` here; nothing could run yt or AMReX against
it.
"""
from __future__ import annotations

import os

import numpy as np

from .problems import NCONS, NGHOST

STATE_NAMES = ("density", "xmom", "ymom", "zmom", "energy")
DERIVED_NAMES = ("pressure", "temperature", "x_velocity", "y_velocity", "z_velocity")
FAB_REAL = "(8, (64 11 52 0 1 12 0 1023)),(8, (8 7 6 5 4 3 2 1))"  # IEEE double, little-endian


def _g(x):
    return "%.17g" % float(x)


def _box(lo, hi):
    return "((%d,%d,%d) (%d,%d,%d) (0,0,0))" % (lo[0], lo[1], lo[2], hi[0], hi[1], hi[2])


def write_plotfile_data(path, names, boxes, data, dx, prob_lo, domain, time=0.0, step=0):
    """Write one level's plot data: `boxes` a list of (lo, n) with n = (nx,
    ny, nz), `data[b]` a host array (len(names), nz, ny, nx) of float64,
    `domain` the (lo, n) of the level's domain.  Returns the path."""
    names = list(names)
    nvar = len(names)
    if nvar == 0:
        raise ValueError("at least one variable to plot")  # writePlotFile aborts the same way
    dlo, dn = [int(v) for v in domain[0]], [int(v) for v in domain[1]]
    dhi = [dlo[d] + dn[d] - 1 for d in range(3)]
    plo = [float(v) for v in prob_lo]
    phi = [plo[d] + dn[d] * float(dx[d]) for d in range(3)]
    lev_dir = os.path.join(path, "Level_0")
    os.makedirs(lev_dir, exist_ok=True)
    # ---- Header (src/CNS.cpp:689-796)
    h = ["HyperCLaw-V1.1", str(nvar)] + names + ["3", _g(time), "0",
                                                 "".join(_g(v) + " " for v in plo),
                                                 "".join(_g(v) + " " for v in phi),
                                                 "",
                                                 _box(dlo, dhi) + " ",
                                                 "%d " % step,
                                                 "".join(_g(v) + " " for v in dx),
                                                 "0", "0",
                                                 "0 %d %s" % (len(boxes), _g(time)),
                                                 "%d" % step]
    for lo, n in boxes:
        for d in range(3):
            h.append("%s %s" % (_g(plo[d] + (lo[d] - dlo[d]) * float(dx[d])),
                                _g(plo[d] + (lo[d] - dlo[d] + n[d]) * float(dx[d]))))
    h.append("Level_0/Cell")
    with open(os.path.join(path, "Header"), "w") as f:
        f.write("\n".join(h) + "\n")
    # ---- Level_0/Cell_D_00000: the FABs one after another
    offsets, mins, maxs = [], [], []
    with open(os.path.join(lev_dir, "Cell_D_00000"), "wb") as f:
        for (lo, n), a in zip(boxes, data):
            a = np.ascontiguousarray(a, dtype="<f8")
            if a.shape != (nvar, n[2], n[1], n[0]):
                raise ValueError("plot data of box %s has shape %s" % (lo, a.shape))
            hi = [lo[d] + n[d] - 1 for d in range(3)]
            offsets.append(f.tell())
            f.write(("FAB (%s)%s %d\n" % (FAB_REAL, _box(lo, hi), nvar)).encode())
            f.write(a.tobytes())
            flat = a.reshape(nvar, -1)
            mins.append(flat.min(axis=1))
            maxs.append(flat.max(axis=1))
    # ---- Level_0/Cell_H: VisMF header
    c = ["1", "1", str(nvar), "0", "(%d 0" % len(boxes)]
    for lo, n in boxes:
        c.append(_box(lo, [lo[d] + n[d] - 1 for d in range(3)]))
    c.append(")")
    c.append(str(len(boxes)))
    c += ["FabOnDisk: Cell_D_00000 %d" % o for o in offsets]
    c.append("")
    for vals in (mins, maxs):
        c.append("%d,%d" % (len(boxes), nvar))
        c += ["".join("%.16e," % v for v in m) for m in vals]
        c.append("")
    with open(os.path.join(lev_dir, "Cell_H"), "w") as f:
        f.write("\n".join(c) + "\n")
    return path


def write_plotfile(path, boxes, states, closures, dx, prob_lo, domain, time=0.0, step=0, derive=DERIVED_NAMES,
                   ng=NGHOST):
    """Plotfile of a level of boxes whose states are cuda tensors (5 + ghosts,
    ghost depth `ng`): the state components and the derived quantities
    `derive` (a subset of DERIVED_NAMES, amr.derive_plot_vars; written in the
    order the reference registers them), derived on the device."""
    import torch

    from . import capi
    sel = [k for k, name in enumerate(DERIVED_NAMES) if name in set(derive)]
    unknown = set(derive) - set(DERIVED_NAMES)
    if unknown:
        raise ValueError("unknown derived variables: %s" % sorted(unknown))
    data = []
    for (lo, n), U in zip(boxes, states):
        der = torch.empty((5, n[2], n[1], n[0]), dtype=torch.float64, device=U.device)
        capi.plot_derive(closures, U, lo, der, ng=ng)
        g = ng
        valid = U[:, g:U.shape[1] - g, g:U.shape[2] - g, g:U.shape[3] - g] if g else U
        data.append(torch.cat([valid[:NCONS], der[sel]]).cpu().numpy())
    names = list(STATE_NAMES) + [DERIVED_NAMES[k] for k in sel]
    return write_plotfile_data(path, names, boxes, data, dx, prob_lo, domain, time, step)


def read_plotfile(path):
    """Read a single-level plotfile written as above: a dict with the
    variable names, time, step, problem extent, domain, cell sizes, the
    boxes (lo, hi) and one (nvar, nz, ny, nx) array per box."""
    with open(os.path.join(path, "Header")) as f:
        lines = f.read().split("\n")
    if lines[0] != "HyperCLaw-V1.1":
        raise ValueError("not a plotfile Header")
    nvar = int(lines[1])
    names = lines[2:2 + nvar]
    p = 2 + nvar
    out = {"names": names, "dim": int(lines[p]), "time": float(lines[p + 1]), "finest_level": int(lines[p + 2]),
           "prob_lo": [float(v) for v in lines[p + 3].split()], "prob_hi": [float(v) for v in lines[p + 4].split()],
           "ref_ratios": lines[p + 5], "domain": lines[p + 6].strip(), "step": int(lines[p + 7]),
           "dx": [float(v) for v in lines[p + 8].split()], "coord": int(lines[p + 9]),
           "bndry": int(lines[p + 10])}
    lev = lines[p + 11].split()
    nbox = int(lev[1])
    out["level_time"] = float(lev[2])
    out["level_step"] = int(lines[p + 12])
    out["grid_extents"] = [[float(v) for v in lines[p + 13 + 3 * b + d].split()] for b in range(nbox) for d in range(3)]
    out["path"] = lines[p + 13 + 3 * nbox]
    with open(os.path.join(path, "Level_0", "Cell_H")) as f:
        ch = f.read().split("\n")
    fods = [ln.split() for ln in ch if ln.startswith("FabOnDisk:")]
    boxes, data = [], []
    with open(os.path.join(path, "Level_0", "Cell_D_00000"), "rb") as f:
        raw = f.read()
    for _, fname, off in fods:
        off = int(off)
        end = raw.index(b"\n", off)
        head = raw[off:end].decode()
        bpart = head[head.index(")((") + 1:head.rindex(")") + 1]
        nums = [int(v) for v in bpart.replace("(", " ").replace(")", " ").replace(",", " ").split()]
        lo, hi = nums[0:3], nums[3:6]
        nc = int(head.split()[-1])
        n = [hi[d] - lo[d] + 1 for d in range(3)]
        cnt = nc * n[0] * n[1] * n[2]
        a = np.frombuffer(raw, dtype="<f8", count=cnt, offset=end + 1).reshape(nc, n[2], n[1], n[0])
        boxes.append((lo, hi))
        data.append(a.copy())
    out["boxes"], out["data"] = boxes, data
    return out
