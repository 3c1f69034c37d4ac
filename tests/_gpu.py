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
                courant_num=float(m["cfl"]), freestream_mach=tuple(m["mach"]))


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def hist_rel_err(h, ref):
    return np.max(np.abs(h - ref) / np.maximum(np.abs(ref), 1e-300))
