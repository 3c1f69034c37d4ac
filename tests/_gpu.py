"""Shared helpers of the GPU parity tests."""
import numpy as np

from bes_gb300 import build as nbuild
from bes_gb300 import lib


def context(mesh, **opts):
    nbuild.build()
    o = lib.default_options(**opts)
    return lib.Context(mesh, o)


def explicit_opts(info):
    m = info["meta"]
    return dict(solver_type=0, local_time_step=1 if m["local"] == "YES" else 0,
                courant_num=float(m["cfl"]), freestream_mach=tuple(m["mach"]),
                freestream_ramp=int(m.get("fs_ramp", 0)),
                freestream_ramp_start_frac=float(m.get("fs_frac", 0.5)))


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def hist_rel_err(h, ref, floor=1e-4):
    """Largest relative difference of two norm histories ([steps, k]).  Each entry is compared
    relative to itself, but never to less than `floor` times the largest norm of the same
    group of five (L2 or max) in that step: a variable whose residual is pure rounding noise
    (e.g. the spanwise momentum of a 2-D flow) has no meaningful relative error."""
    h = np.asarray(h, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.abs(ref).copy()
    for g0 in range(0, min(ref.shape[1], 10), 5):
        grp = np.abs(ref[:, g0:g0 + 5]).max(axis=1, keepdims=True)
        scale[:, g0:g0 + 5] = np.maximum(scale[:, g0:g0 + 5], floor * grp)
    return np.max(np.abs(h - ref) / np.maximum(scale, 1e-300))
