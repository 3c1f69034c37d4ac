"""ctypes access to the CPU restatement (oracle/bes_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of bench.py, as the checker.  The product never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libbes_oracle.so")
SOURCES = [os.path.join(HERE, "bes_oracle.cpp"), os.path.join(HERE, "bes_oracle.hpp"),
           os.path.join(HERE, "linsolve.hpp")]


def build(force: bool = False) -> str:
    """Compile the restatement with g++ (no FMA contraction, so x86 and Arm agree)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH):
        lib_t = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(s) <= lib_t for s in SOURCES):
            return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           os.path.join(HERE, "bes_oracle.cpp"), "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


class _Opts(ctypes.Structure):
    _fields_ = [
        ("solver", ctypes.c_int32), ("local_dt", ctypes.c_int32), ("n_stage", ctypes.c_int32),
        ("muscl_exact", ctypes.c_int32), ("jacobian_repeat", ctypes.c_int32),
        ("lin_precond", ctypes.c_int32), ("lin_restart", ctypes.c_int32),
        ("lin_maxiter", ctypes.c_int32), ("ramp_steps", ctypes.c_int32),
        ("threads", ctypes.c_int32), ("pad0", ctypes.c_int32), ("pad1", ctypes.c_int32),
        ("cfl", ctypes.c_double), ("cfl_max", ctypes.c_double), ("cfl_exp0", ctypes.c_double),
        ("cfl_exp1", ctypes.c_double), ("alpha", ctypes.c_double * 8),
        ("venkat_k", ctypes.c_double), ("harten", ctypes.c_double),
        ("gas_constant", ctypes.c_double), ("gamma", ctypes.c_double),
        ("mach", ctypes.c_double * 3), ("lin_tol", ctypes.c_double),
        ("ramp_cfl0", ctypes.c_double), ("ramp_cfl1", ctypes.c_double),
        ("fs_ramp", ctypes.c_int32), ("pad2", ctypes.c_int32), ("fs_frac", ctypes.c_double),
    ]


DEFAULTS = dict(solver=0, local_dt=1, n_stage=4, muscl_exact=0, jacobian_repeat=0,
                lin_precond=0, lin_restart=30, lin_maxiter=1000, ramp_steps=0, threads=1,
                cfl=0.8, cfl_max=0.0, cfl_exp=(1.0, 1.0),
                alpha=(0.0833, 0.2069, 0.4265, 1.0), venkat_k=5.0, harten=0.05,
                gas_constant=287.0, gamma=1.4, mach=(0.5, 0.0, 0.0), lin_tol=1e-7,
                ramp_cfl0=0.0, ramp_cfl1=0.0, fs_ramp=0, fs_frac=0.5)

_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        D = ctypes.POINTER(ctypes.c_double)
        I64 = ctypes.POINTER(ctypes.c_int64)
        L.bor_create.restype = P
        L.bor_create.argtypes = [D, ctypes.c_int64, I64, ctypes.c_int64, I64,
                                 ctypes.POINTER(ctypes.c_int32), ctypes.c_int64, ctypes.c_int32,
                                 ctypes.POINTER(_Opts), ctypes.c_char_p]
        L.bor_destroy.argtypes = [P]
        L.bor_sizes.argtypes = [P, I64]
        L.bor_geometry.argtypes = [P, D, D, D, D, I64, I64, D, D, D, D, I64, I64, I64, I64]
        L.bor_set_state.argtypes = [P, D]
        L.bor_get_state.argtypes = [P, D]
        L.bor_operators.argtypes = [P, ctypes.c_double, D, D, D, D, D, D, D]
        L.bor_explicit_run.argtypes = [P, ctypes.c_int64, D]
        L.bor_implicit_run.argtypes = [P, ctypes.c_int64, D]
        L.bor_set_ilu_order.argtypes = [P, I64]
        L.bor_set_ilu_domain.argtypes = [P, I64]
        L.bor_implicit_assemble.restype = ctypes.c_int64
        L.bor_implicit_assemble.argtypes = [P, ctypes.c_double, D, D, I64, I64]
        L.bor_flux_batch.argtypes = [P, ctypes.c_int32, ctypes.c_int64, D, D, D, D, D, D]
        L.bor_pinf.argtypes = [P, D]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _i(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)) if a is not None else None


def make_opts(**kw) -> _Opts:
    cfg = dict(DEFAULTS)
    cfg.update(kw)
    o = _Opts()
    for k in ("solver", "local_dt", "n_stage", "muscl_exact", "jacobian_repeat", "lin_precond",
              "lin_restart", "lin_maxiter", "ramp_steps", "threads", "fs_ramp"):
        setattr(o, k, int(cfg[k]))
    for k in ("cfl", "cfl_max", "venkat_k", "harten", "gas_constant", "gamma", "lin_tol",
              "ramp_cfl0", "ramp_cfl1", "fs_frac"):
        setattr(o, k, float(cfg[k]))
    o.cfl_exp0, o.cfl_exp1 = (float(x) for x in cfg["cfl_exp"])
    al = list(cfg["alpha"]) + [0.0] * (8 - len(cfg["alpha"]))
    for i in range(8):
        o.alpha[i] = al[i]
    o.n_stage = len(cfg["alpha"])
    for i in range(3):
        o.mach[i] = float(cfg["mach"][i])
    return o


class Oracle:
    """One mesh + options; state kept in reference (file) numbering, cell-major AoS [nc,5]."""

    def __init__(self, mesh, **opts):
        """mesh: tetrahedra [nc,4] with boundary triangles [nb,3], or triangles [nc,3] with
        boundary lines [nb,2] (the reference's 2-D path)."""
        L = lib()
        self._keep = [np.ascontiguousarray(mesh.nodes, dtype=np.float64),
                      np.ascontiguousarray(mesh.tets, dtype=np.int64),
                      np.ascontiguousarray(mesh.btris, dtype=np.int64),
                      np.ascontiguousarray(mesh.btags, dtype=np.int32)]
        nodes, tets, btris, btags = self._keep
        self.opts = make_opts(**opts)
        err = ctypes.create_string_buffer(256)
        self.h = L.bor_create(_d(nodes), nodes.shape[0], _i(tets), tets.shape[0], _i(btris),
                              btags.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                              btris.shape[0], 2 if tets.shape[1] == 3 else 3,
                              ctypes.byref(self.opts), err)
        if not self.h:
            raise ValueError("oracle mesh build failed: " + err.value.decode())
        sz = np.zeros(2, dtype=np.int64)
        L.bor_sizes(self.h, _i(sz))
        self.nc, self.nf = int(sz[0]), int(sz[1])

    def __del__(self):
        if getattr(self, "h", None):
            lib().bor_destroy(self.h)
            self.h = None

    def geometry(self) -> dict:
        nc, nf = self.nc, self.nf
        g = dict(volume=np.zeros(nc), centroid=np.zeros((nc, 3)), vec_to_face=np.zeros((nc, 4, 3)),
                 weight=np.zeros((nc, 4)), cell_face=np.zeros((nc, 4), np.int64),
                 cell_adj=np.zeros((nc, 4), np.int64), face_S=np.zeros((nf, 3)),
                 face_n=np.zeros((nf, 3)), face_area=np.zeros(nf), face_center=np.zeros((nf, 3)),
                 face_owner=np.zeros(nf, np.int64), face_neigh=np.zeros(nf, np.int64),
                 face_type=np.zeros(nf, np.int64), muscl_slot=np.zeros((nc, 4), np.int64))
        lib().bor_geometry(self.h, _d(g["volume"]), _d(g["centroid"]), _d(g["vec_to_face"]),
                           _d(g["weight"]), _i(g["cell_face"]), _i(g["cell_adj"]),
                           _d(g["face_S"]), _d(g["face_n"]), _d(g["face_area"]),
                           _d(g["face_center"]), _i(g["face_owner"]), _i(g["face_neigh"]),
                           _i(g["face_type"]), _i(g["muscl_slot"]))
        return g

    def set_state(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(self.nc, 5)
        lib().bor_set_state(self.h, _d(U))

    def get_state(self):
        U = np.zeros((self.nc, 5))
        lib().bor_get_state(self.h, _d(U))
        return U

    def operators(self, cfl: float) -> dict:
        nc, nf = self.nc, self.nf
        o = dict(dt=np.zeros(nc), grad=np.zeros((nc, 5, 3)), limiter=np.zeros((nc, 5)),
                 face_UL=np.zeros((nf, 5)), face_UR=np.zeros((nf, 5)), face_flux=np.zeros((nf, 5)),
                 residual=np.zeros((nc, 5)))
        lib().bor_operators(self.h, float(cfl), _d(o["dt"]), _d(o["grad"]), _d(o["limiter"]),
                            _d(o["face_UL"]), _d(o["face_UR"]), _d(o["face_flux"]),
                            _d(o["residual"]))
        return o

    def explicit_run(self, n: int) -> np.ndarray:
        h = np.zeros((n, 10))
        lib().bor_explicit_run(self.h, int(n), _d(h))
        return h

    def set_ilu_order(self, order):
        order = np.ascontiguousarray(order, dtype=np.int64)
        lib().bor_set_ilu_order(self.h, _i(order))

    def set_ilu_domain(self, dom):
        """Subdomain id per cell (reference numbering); couplings between subdomains are left
        out of the block-ILU(0) preconditioner.  None restores the global factorisation."""
        d = None if dom is None else np.ascontiguousarray(dom, dtype=np.int64)
        lib().bor_set_ilu_domain(self.h, _i(d))

    def implicit_run(self, n: int) -> np.ndarray:
        h = np.zeros((n, 19))
        lib().bor_implicit_run(self.h, int(n), _d(h))
        return h

    def implicit_assemble(self, cfl: float) -> dict:
        nc = self.nc
        nblk = lib().bor_implicit_assemble(self.h, float(cfl), None, None, None, None)
        out = dict(rhs=np.zeros((nc, 5)), vals=np.zeros((nblk, 5, 5)),
                   rowptr=np.zeros(nc + 1, np.int64), col=np.zeros(nblk, np.int64))
        lib().bor_implicit_assemble(self.h, float(cfl), _d(out["rhs"]), _d(out["vals"]),
                                    _i(out["rowptr"]), _i(out["col"]))
        return out

    def flux_batch(self, kind: int, UL, UR, nhat, jacobians: bool = False):
        UL = np.ascontiguousarray(UL, dtype=np.float64)
        UR = np.ascontiguousarray(UR, dtype=np.float64)
        nhat = np.ascontiguousarray(nhat, dtype=np.float64)
        n = UL.shape[0]
        F = np.zeros((n, 5))
        JL = np.zeros((n, 5, 5)) if jacobians else None
        JR = np.zeros((n, 5, 5)) if (jacobians and kind == 0) else None
        lib().bor_flux_batch(self.h, int(kind), n, _d(UL), _d(UR), _d(nhat), _d(F), _d(JL),
                             _d(JR))
        return (F, JL, JR) if jacobians else F

    def pinf(self):
        p = np.zeros(6)
        lib().bor_pinf(self.h, _d(p))
        return p
