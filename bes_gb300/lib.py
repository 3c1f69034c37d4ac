"""ctypes binding of libbes_gb300.so (include/bes_gb300.h) and a small Python mirror of the
reference's solver interface (Solver::initialize / setUniversalInitialCondition / solve).

The native library is required: every call goes to the sm_103a CUDA path and fails loudly if
the library or a GPU is missing.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libbes_gb300.so")

BES_OK = 0
ERRORS = {1: "BES_ERR_INVALID", 2: "BES_ERR_CUDA", 3: "BES_ERR_NAN", 4: "BES_ERR_MESH",
          5: "BES_ERR_CONFIG", 6: "BES_ERR_UNSUPPORTED", 7: "BES_ERR_TIMEOUT"}

# every extern "C" symbol declared in include/bes_gb300.h
EXPORTED = [
    "bes_options_default", "bes_options_from_besi", "bes_mesh_read_gmsh", "bes_mesh_free",
    "bes_create", "bes_destroy", "bes_last_error", "bes_sizes", "bes_set_freestream_state",
    "bes_set_state", "bes_get_state", "bes_compute_operators", "bes_explicit_iterations",
    "bes_flux_batch", "bes_build_info", "bes_abi_sizes", "bes_host_geometry",
    "bes_explicit_enqueue", "bes_synchronize", "bes_stream", "bes_last_kernel_times",
    "bes_residual_norms_static", "bes_implicit_steps", "bes_implicit_assemble",
    "bes_ilu_order", "bes_counters", "bes_wall_force", "bes_profile",
    "bes_output_default", "bes_output_from_besi", "bes_write", "bes_write_host", "bes_solve",
    "bes_create_batch", "bes_conditions", "bes_set_active", "bes_sweep_run",
    "bes_implicit_stats", "bes_set_linear_guard", "bes_set_condition", "bes_implicit_sweep",
    "bes_tuning", "bes_fp64_fma_rate", "bes_host_layout_digest", "bes_checkpoint_save",
    "bes_checkpoint_load",
    "bes_mlp_create", "bes_mlp_destroy", "bes_mlp_last_error", "bes_mlp_train", "bes_mlp_infer",
    "bes_mlp_init_state", "bes_mlp_params", "bes_mlp_features", "bes_mlp_loss_grad",
    "bes_mlp_apply_grad", "bes_mlp_normalisation",
]

OUTPUT_VTK, OUTPUT_CSV, OUTPUT_SLIP_WALL_CSV = 0, 1, 2


class BesError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class MeshArrays(ctypes.Structure):
    _fields_ = [("n_nodes", ctypes.c_int64), ("nodes", ctypes.POINTER(ctypes.c_double)),
                ("n_btris", ctypes.c_int64), ("btris", ctypes.POINTER(ctypes.c_int64)),
                ("btags", ctypes.POINTER(ctypes.c_int32)), ("n_tets", ctypes.c_int64),
                ("tets", ctypes.POINTER(ctypes.c_int64)), ("dim", ctypes.c_int32)]


class Output(ctypes.Structure):
    """bes_output: the .besi output keys."""
    _fields_ = [("folder", ctypes.c_char * 1024), ("format", ctypes.c_int32),
                ("slip_wall", ctypes.c_int32), ("save_interval", ctypes.c_int64),
                ("verbose", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class Options(ctypes.Structure):
    _fields_ = [
        ("solver_type", ctypes.c_int32), ("local_time_step", ctypes.c_int32),
        ("n_stage", ctypes.c_int32), ("muscl_face_vector", ctypes.c_int32),
        ("stage_coeff", ctypes.c_double * 8), ("courant_num", ctypes.c_double),
        ("adaptive_courant_num_max", ctypes.c_double),
        ("adaptive_courant_num_exponent", ctypes.c_double * 2),
        ("venkatakrishnan_factor", ctypes.c_double), ("harten_correction_limit", ctypes.c_double),
        ("gas_constant", ctypes.c_double), ("specific_heat_ratio", ctypes.c_double),
        ("freestream_mach", ctypes.c_double * 3), ("number_of_time_step", ctypes.c_int32),
        ("linear_solver", ctypes.c_int32), ("linear_solver_max_iter", ctypes.c_int32),
        ("gmres_restart", ctypes.c_int32), ("linear_solver_tol", ctypes.c_double),
        ("jacobian_repeat", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("cfl_ramp_steps", ctypes.c_int32), ("freestream_ramp", ctypes.c_int32),
        ("cfl_ramp_start", ctypes.c_double), ("cfl_ramp_end", ctypes.c_double),
        ("freestream_ramp_start_frac", ctypes.c_double), ("sweep_kernel", ctypes.c_int32),
        ("reserved_i", ctypes.c_int32), ("reserved", ctypes.c_double * 2),
    ]


_lib = None


def load(path: str = LIB_PATH):
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"native library missing: {path} (run python -m bes_gb300.build)")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    D = ctypes.POINTER(ctypes.c_double)
    L.bes_options_default.argtypes = [ctypes.POINTER(Options)]
    L.bes_options_from_besi.argtypes = [ctypes.c_char_p, ctypes.POINTER(Options), ctypes.c_char_p,
                                        ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t]
    L.bes_mesh_read_gmsh.argtypes = [ctypes.c_char_p, ctypes.POINTER(MeshArrays),
                                     ctypes.c_char_p, ctypes.c_size_t]
    L.bes_mesh_free.argtypes = [ctypes.POINTER(MeshArrays)]
    L.bes_create.argtypes = [ctypes.POINTER(MeshArrays), ctypes.POINTER(Options),
                             ctypes.POINTER(P)]
    L.bes_destroy.argtypes = [P]
    L.bes_last_error.argtypes = [P]
    L.bes_last_error.restype = ctypes.c_char_p
    L.bes_sizes.argtypes = [P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    L.bes_set_freestream_state.argtypes = [P]
    L.bes_set_state.argtypes = [P, D]
    L.bes_get_state.argtypes = [P, D]
    L.bes_compute_operators.argtypes = [P, ctypes.c_double, D, D, D, D, D, D, D]
    L.bes_explicit_iterations.argtypes = [P, ctypes.c_int64, D]
    L.bes_flux_batch.argtypes = [P, ctypes.c_int32, ctypes.c_int64, D, D, D, D, D, D]
    L.bes_build_info.restype = ctypes.c_char_p
    L.bes_abi_sizes.argtypes = [ctypes.POINTER(ctypes.c_int64)]
    L.bes_explicit_enqueue.argtypes = [P, ctypes.c_int64]
    L.bes_synchronize.argtypes = [P]
    L.bes_stream.argtypes = [P]
    L.bes_stream.restype = ctypes.c_void_p
    L.bes_last_kernel_times.argtypes = [P, D]
    L.bes_implicit_steps.argtypes = [P, ctypes.c_int64, D]
    L.bes_implicit_assemble.argtypes = [P, ctypes.c_double, D, D, ctypes.POINTER(ctypes.c_int64)]
    L.bes_ilu_order.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    L.bes_counters.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    L.bes_wall_force.argtypes = [P, D]
    L.bes_profile.argtypes = [P, ctypes.c_int32, D, ctypes.POINTER(ctypes.c_int64)]
    L.bes_residual_norms_static.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
    L.bes_output_default.argtypes = [ctypes.POINTER(Output)]
    L.bes_output_default.restype = None
    L.bes_output_from_besi.argtypes = [ctypes.c_char_p, ctypes.POINTER(Output), ctypes.c_char_p,
                                       ctypes.c_size_t]
    L.bes_write.argtypes = [P, ctypes.c_char_p, ctypes.c_int32]
    L.bes_write_host.argtypes = [ctypes.POINTER(MeshArrays), ctypes.POINTER(Options), D,
                                 ctypes.c_char_p, ctypes.c_int32, ctypes.c_char_p,
                                 ctypes.c_size_t]
    L.bes_solve.argtypes = [P, ctypes.POINTER(Output)]
    L.bes_create_batch.argtypes = [ctypes.POINTER(MeshArrays), ctypes.POINTER(Options),
                                   ctypes.c_int32, D, ctypes.POINTER(P)]
    L.bes_conditions.argtypes = [P, ctypes.POINTER(ctypes.c_int32)]
    L.bes_set_active.argtypes = [P, ctypes.POINTER(ctypes.c_int32)]
    L.bes_sweep_run.argtypes = [P, ctypes.c_int64, ctypes.c_double, ctypes.c_int64,
                                ctypes.POINTER(ctypes.c_int64), D]
    L.bes_implicit_stats.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    L.bes_set_linear_guard.argtypes = [P, ctypes.c_int32]
    L.bes_tuning.argtypes = [P, ctypes.c_char_p, ctypes.c_size_t]
    L.bes_fp64_fma_rate.argtypes = [D]
    L.bes_checkpoint_save.argtypes = [P, ctypes.c_char_p]
    L.bes_checkpoint_load.argtypes = [P, ctypes.c_char_p]
    L.bes_host_layout_digest.argtypes = [ctypes.POINTER(MeshArrays), ctypes.c_int32,
                                         ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64),
                                         ctypes.c_int32, ctypes.POINTER(ctypes.c_int32),
                                         ctypes.c_char_p, ctypes.c_size_t]
    L.bes_set_condition.argtypes = [P, ctypes.c_int32, D, D]
    L.bes_implicit_sweep.argtypes = [P, ctypes.c_int32, D, D, D, ctypes.c_double, ctypes.c_int64,
                                     ctypes.POINTER(ctypes.c_int64), D, D, D, D]
    F32 = ctypes.POINTER(ctypes.c_float)
    I64p = ctypes.POINTER(ctypes.c_int64)
    L.bes_mlp_create.argtypes = [P, ctypes.c_uint64, ctypes.POINTER(P)]
    L.bes_mlp_destroy.argtypes = [P]
    L.bes_mlp_destroy.restype = None
    L.bes_mlp_last_error.argtypes = [P]
    L.bes_mlp_last_error.restype = ctypes.c_char_p
    L.bes_mlp_train.argtypes = [P, ctypes.c_int32, D, D, ctypes.c_int64, ctypes.c_int32,
                                ctypes.c_double, ctypes.c_double, ctypes.c_uint64, D]
    L.bes_mlp_infer.argtypes = [P, ctypes.c_int32, D, D]
    L.bes_mlp_init_state.argtypes = [P, P, ctypes.POINTER(ctypes.c_int32)]
    L.bes_mlp_params.argtypes = [P, F32, F32, I64p]
    L.bes_mlp_features.argtypes = [P, F32]
    L.bes_mlp_loss_grad.argtypes = [P, ctypes.c_int32, I64p, D, D, D, F32, D]
    L.bes_mlp_apply_grad.argtypes = [P, F32, ctypes.c_double, ctypes.c_double]
    L.bes_mlp_normalisation.argtypes = [P, D]
    I64 = ctypes.POINTER(ctypes.c_int64)
    L.bes_host_geometry.argtypes = [ctypes.POINTER(MeshArrays), ctypes.c_int32, I64, I64, D, D, D,
                                    D, I64, I64, I64, I64, I64, I64, ctypes.c_char_p,
                                    ctypes.c_size_t]
    for name in EXTRA_SIGNATURES:
        fn = getattr(L, name, None)
        if fn is not None:
            fn.argtypes, fn.restype = EXTRA_SIGNATURES[name]
    _lib = L
    return L


EXTRA_SIGNATURES: dict = {}


def _d(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def default_options(**kw) -> Options:
    o = Options()
    load().bes_options_default(ctypes.byref(o))
    for k, v in kw.items():
        if k in ("stage_coeff",):
            o.n_stage = len(v)
            for i, x in enumerate(v):
                o.stage_coeff[i] = float(x)
        elif k in ("freestream_mach", "adaptive_courant_num_exponent"):
            arr = getattr(o, k)
            for i, x in enumerate(v):
                arr[i] = float(x)
        else:
            setattr(o, k, v)
    return o


def options_from_besi(path: str) -> tuple[Options, str]:
    o = Options()
    mesh = ctypes.create_string_buffer(4096)
    err = ctypes.create_string_buffer(512)
    rc = load().bes_options_from_besi(path.encode(), ctypes.byref(o), mesh, 4096, err, 512)
    if rc != BES_OK:
        raise BesError(rc, err.value.decode())
    return o, mesh.value.decode()


def default_output(**kw) -> Output:
    """bes_output with the reference's defaults; keyword arguments override fields."""
    o = Output()
    load().bes_output_default(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v.encode() if k == "folder" else v)
    return o


def output_from_besi(path: str) -> Output:
    o = Output()
    err = ctypes.create_string_buffer(512)
    rc = load().bes_output_from_besi(path.encode(), ctypes.byref(o), err, 512)
    if rc != BES_OK:
        raise BesError(rc, err.value.decode())
    return o


def write_host(mesh, options: Options, U, path: str, kind: int = OUTPUT_VTK):
    """bes_write_host: the reference's output file for state U [n_cells][5] (reference
    numbering), on the host (no GPU)."""
    keep = _MeshKeep(mesh)
    U = np.ascontiguousarray(U, dtype=np.float64)
    err = ctypes.create_string_buffer(512)
    rc = load().bes_write_host(ctypes.byref(keep.c), ctypes.byref(options), _d(U),
                               path.encode(), int(kind), err, 512)
    if rc != BES_OK:
        raise BesError(rc, err.value.decode())


def residual_norms_static(residual_ptr: int, n_cells: int, norms_ptr: int, stream: int = 0):
    """bes_residual_norms_static on device pointers (no allocation inside the library)."""
    err = ctypes.create_string_buffer(256)
    rc = load().bes_residual_norms_static(ctypes.c_void_p(residual_ptr), int(n_cells),
                                          ctypes.c_void_p(norms_ptr), ctypes.c_void_p(stream),
                                          err, 256)
    if rc != BES_OK:
        raise BesError(rc, err.value.decode())


class _MeshKeep:
    """Keeps numpy arrays alive for a MeshArrays view."""

    def __init__(self, mesh):
        self.nodes = np.ascontiguousarray(mesh.nodes, dtype=np.float64)
        self.tets = np.ascontiguousarray(mesh.tets, dtype=np.int64)
        self.btris = np.ascontiguousarray(mesh.btris, dtype=np.int64)
        self.btags = np.ascontiguousarray(mesh.btags, dtype=np.int32)
        self.c = MeshArrays(self.nodes.shape[0], _d(self.nodes), self.btris.shape[0],
                            self.btris.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                            self.btags.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                            self.tets.shape[0],
                            self.tets.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                            2 if self.tets.shape[1] == 3 else 3)


def fp64_fma_rate() -> float:
    """bes_fp64_fma_rate: FP64 FMA per second of the current device."""
    r = ctypes.c_double()
    rc = load().bes_fp64_fma_rate(ctypes.byref(r))
    if rc:
        raise BesError(rc, "bes_fp64_fma_rate failed")
    return r.value


def _i(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def host_layout_digest(mesh, muscl_exact: bool = False, rcm_ilu_order: bool = False) -> list:
    """bes_host_layout_digest: 64-bit digests of every device-layout array of the mesh build."""
    L = load()
    keep = _MeshKeep(mesh)
    n = ctypes.c_int32()
    err = ctypes.create_string_buffer(512)
    out = (ctypes.c_uint64 * 64)()
    rc = L.bes_host_layout_digest(ctypes.byref(keep.c), int(muscl_exact), int(rcm_ilu_order),
                                  out, 64, ctypes.byref(n), err, 512)
    if rc != BES_OK:
        raise BesError(rc, err.value.decode())
    return [int(out[i]) for i in range(n.value)]


def host_geometry(mesh, muscl_exact: bool = False) -> dict:
    """The library's host-side mesh build (no GPU), in reference numbering."""
    L = load()
    keep = _MeshKeep(mesh)
    nc, nf = ctypes.c_int64(), ctypes.c_int64()
    err = ctypes.create_string_buffer(512)
    rc = L.bes_host_geometry(ctypes.byref(keep.c), int(muscl_exact), ctypes.byref(nc),
                             ctypes.byref(nf), None, None, None, None, None, None, None, None,
                             None, None, err, 512)
    if rc != BES_OK:
        raise BesError(rc, err.value.decode())
    nc, nf = nc.value, nf.value
    g = dict(volume=np.zeros(nc), centroid=np.zeros((nc, 3)), face_S=np.zeros((nf, 3)),
             face_area=np.zeros(nf), face_owner=np.zeros(nf, np.int64),
             face_neigh=np.zeros(nf, np.int64), face_type=np.zeros(nf, np.int64),
             muscl_slot=np.zeros((nc, 4), np.int64), cell_new2ref=np.zeros(nc, np.int64),
             face_new2ref=np.zeros(nf, np.int64))
    rc = L.bes_host_geometry(ctypes.byref(keep.c), int(muscl_exact), None, None,
                             _d(g["volume"]), _d(g["centroid"]), _d(g["face_S"]),
                             _d(g["face_area"]), _i(g["face_owner"]), _i(g["face_neigh"]),
                             _i(g["face_type"]), _i(g["muscl_slot"]), _i(g["cell_new2ref"]),
                             _i(g["face_new2ref"]), err, 512)
    if rc != BES_OK:
        raise BesError(rc, err.value.decode())
    return g


def read_gmsh(path: str):
    """Gmsh 2.2 file -> meshgen.TetMesh-like arrays through the library's reader."""
    from .meshgen import TetMesh
    L = load()
    m = MeshArrays()
    err = ctypes.create_string_buffer(512)
    rc = L.bes_mesh_read_gmsh(path.encode(), ctypes.byref(m), err, 512)
    if rc != BES_OK:
        raise BesError(rc, err.value.decode())
    try:
        nd = 2 if m.dim == 2 else 3
        nodes = np.ctypeslib.as_array(m.nodes, shape=(m.n_nodes, 3)).copy()
        tets = np.ctypeslib.as_array(m.tets, shape=(m.n_tets, nd + 1)).copy()
        if m.n_btris:
            btris = np.ctypeslib.as_array(m.btris, shape=(m.n_btris, nd)).copy()
            btags = np.ctypeslib.as_array(m.btags, shape=(m.n_btris,)).copy().astype(np.int64)
        else:
            btris = np.zeros((0, nd), np.int64)
            btags = np.zeros(0, np.int64)
    finally:
        L.bes_mesh_free(ctypes.byref(m))
    return TetMesh(nodes, tets, btris, btags, name=os.path.basename(path))


class Context:
    """One mesh + options on the current CUDA device (the reference's Solver objects).  With
    `machs` ([n_cond][3]) the context holds a batch of freestream conditions
    (bes_create_batch); state, histories and forces then carry a leading condition axis."""

    def __init__(self, mesh, options: Options, machs=None):
        L = load()
        self._mesh = _MeshKeep(mesh)
        self.options = options
        h = ctypes.c_void_p()
        if machs is None:
            self.n_cond = 1
            self.batched = False
            rc = L.bes_create(ctypes.byref(self._mesh.c), ctypes.byref(options), ctypes.byref(h))
        else:
            m = np.ascontiguousarray(machs, dtype=np.float64).reshape(-1, 3)
            self.n_cond = m.shape[0]
            self.batched = True
            rc = L.bes_create_batch(ctypes.byref(self._mesh.c), ctypes.byref(options),
                                    self.n_cond, _d(m), ctypes.byref(h))
        if rc != BES_OK:
            raise BesError(rc, "bes_create failed (mesh, options or CUDA device)")
        self.h = h
        nc, nf = ctypes.c_int64(), ctypes.c_int64()
        L.bes_sizes(self.h, ctypes.byref(nc), ctypes.byref(nf))
        self.n_cells, self.n_faces = nc.value, nf.value

    def _check(self, rc):
        if rc != BES_OK:
            raise BesError(rc, load().bes_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            load().bes_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_freestream_state(self):
        self._check(load().bes_set_freestream_state(self.h))

    def _shape(self, *tail):
        return ((self.n_cond,) if self.batched else ()) + tail

    def set_state(self, U):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(self.n_cond * self.n_cells, 5)
        self._check(load().bes_set_state(self.h, _d(U)))

    def get_state(self) -> np.ndarray:
        U = np.zeros(self._shape(self.n_cells, 5))
        self._check(load().bes_get_state(self.h, _d(U)))
        return U

    def operators(self, cfl: float) -> dict:
        nc, nf = self.n_cells, self.n_faces
        o = dict(dt=np.zeros(nc), grad=np.zeros((nc, 5, 3)), limiter=np.zeros((nc, 5)),
                 face_UL=np.zeros((nf, 5)), face_UR=np.zeros((nf, 5)), face_flux=np.zeros((nf, 5)),
                 residual=np.zeros((nc, 5)))
        self._check(load().bes_compute_operators(
            self.h, float(cfl), _d(o["dt"]), _d(o["grad"]), _d(o["limiter"]), _d(o["face_UL"]),
            _d(o["face_UR"]), _d(o["face_flux"]), _d(o["residual"])))
        return o

    def explicit_iterations(self, n: int, history: bool = True):
        h = np.zeros((n,) + self._shape(10)) if history else None
        self._check(load().bes_explicit_iterations(self.h, int(n), _d(h)))
        return h

    def enqueue(self, n: int):
        """Enqueue n explicit iterations without waiting."""
        self._check(load().bes_explicit_enqueue(self.h, int(n)))

    def synchronize(self):
        self._check(load().bes_synchronize(self.h))

    @property
    def stream_handle(self) -> int:
        return int(load().bes_stream(self.h))

    def last_kernel_times(self) -> dict:
        ms = np.zeros(4)
        self._check(load().bes_last_kernel_times(self.h, _d(ms)))
        return dict(cell_ms=ms[0], face_ms=ms[1], update_ms=ms[2], total_ms=ms[3])

    def implicit_steps(self, n: int):
        """n implicit steps; history [n, 19], batched [n, n_cond, 19] (see bes_implicit_steps)."""
        h = np.zeros((n,) + self._shape(19))
        self._check(load().bes_implicit_steps(self.h, int(n), _d(h)))
        return h

    def implicit_assemble(self, cfl: float) -> dict:
        nb = ctypes.c_int64()
        self._check(load().bes_implicit_assemble(self.h, float(cfl), None, None, ctypes.byref(nb)))
        rhs = np.zeros((self.n_cells, 5))
        blocks = np.zeros((nb.value, 5, 5))
        self._check(load().bes_implicit_assemble(self.h, float(cfl), _d(rhs), _d(blocks),
                                                 ctypes.byref(nb)))
        return dict(rhs=rhs, blocks=blocks)

    PROFILE_CATEGORIES = ("residual", "jacobian", "assemble", "ilu_factor", "precond",
                          "spmv", "gram_schmidt", "update")

    def profile(self, enable: bool = True) -> dict:
        """Turn implicit-path device timing on/off; returns what accumulated since the last
        call as {category: (ms, count)}."""
        ms = np.zeros(8)
        cnt = np.zeros(8, np.int64)
        self._check(load().bes_profile(self.h, int(enable), _d(ms), _i(cnt)))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(self.PROFILE_CATEGORIES)}

    def write(self, path: str, kind: int = OUTPUT_VTK):
        """bes_write: the reference's output file of the current state."""
        self._check(load().bes_write(self.h, path.encode(), int(kind)))

    def solve(self, output: Output | None = None):
        """bes_solve: number_of_time_step steps with the reference's residual.csv and files."""
        self._check(load().bes_solve(self.h, ctypes.byref(output or default_output())))

    def set_active(self, active):
        a = np.ascontiguousarray(active, dtype=np.int32)
        self._check(load().bes_set_active(self.h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))

    def sweep_run(self, max_iter: int, drop: float = 1e-8, check_every: int = 50):
        """bes_sweep_run: iterate every condition to a residual drop; returns (iterations,
        final relative residual) per condition."""
        it = np.zeros(self.n_cond, np.int64)
        fd = np.zeros(self.n_cond)
        self._check(load().bes_sweep_run(self.h, int(max_iter), float(drop), int(check_every),
                                         _i(it), _d(fd)))
        return it, fd

    def wall_force(self) -> np.ndarray:
        f = np.zeros(self._shape(3))
        self._check(load().bes_wall_force(self.h, _d(f)))
        return f

    def counters(self) -> dict:
        out = np.zeros(5, np.int64)
        self._check(load().bes_counters(self.h, _i(out)))
        return dict(launches=int(out[0]), explicit_iterations=int(out[1]),
                    implicit_steps=int(out[2]), linear_iterations=int(out[3]),
                    gram_schmidt_second_passes=int(out[4]))

    def implicit_stats(self) -> dict:
        """bes_implicit_stats: steps, host synchronisations, Arnoldi steps and restart cycles
        the device ran."""
        out = np.zeros(4, np.int64)
        self._check(load().bes_implicit_stats(self.h, _i(out)))
        return dict(steps=int(out[0]), host_syncs=int(out[1]), arnoldi_steps=int(out[2]),
                    restart_cycles=int(out[3]))

    def checkpoint_save(self, path: str):
        """bes_checkpoint_save: state, controllers and counters to a binary file."""
        self._check(load().bes_checkpoint_save(self.h, path.encode()))

    def checkpoint_load(self, path: str):
        """bes_checkpoint_load: continue from a checkpoint of a context like this one."""
        self._check(load().bes_checkpoint_load(self.h, path.encode()))

    def tuning(self) -> str:
        """bes_tuning: the autotuner's candidates, their device times and its choices."""
        buf = ctypes.create_string_buffer(4096)
        self._check(load().bes_tuning(self.h, buf, len(buf)))
        return buf.value.decode()

    def set_linear_guard(self, max_cycles: int):
        """bes_set_linear_guard: restart-cycle limit of one linear solve (0: default)."""
        self._check(load().bes_set_linear_guard(self.h, int(max_cycles)))

    def set_condition(self, cond: int, mach=None, U=None):
        """bes_set_condition: a new condition (Mach vector, state or freestream) in slot cond."""
        m = None if mach is None else np.ascontiguousarray(mach, dtype=np.float64)
        u = None if U is None else np.ascontiguousarray(U, dtype=np.float64)
        self._check(load().bes_set_condition(self.h, int(cond), None if m is None else _d(m),
                                             None if u is None else _d(u)))

    def implicit_sweep(self, machs, drop: float = 1e-8, max_steps: int = 300, U0=None,
                       target=None, states: bool = False) -> dict:
        """bes_implicit_sweep: solve every condition of `machs` [n, 3] to convergence through
        the context's slots; returns per-condition steps, final relative residual, wall force,
        seconds (and final states when `states`)."""
        m = np.ascontiguousarray(machs, dtype=np.float64).reshape(-1, 3)
        n = m.shape[0]
        u0 = None if U0 is None else np.ascontiguousarray(U0, dtype=np.float64)
        tg = None if target is None else np.ascontiguousarray(target, dtype=np.float64)
        steps = np.zeros(n, np.int64)
        fin = np.zeros(n)
        force = np.zeros((n, 3))
        secs = np.zeros(n)
        U = np.zeros((n, self.n_cells, 5)) if states else None
        self._check(load().bes_implicit_sweep(self.h, n, _d(m), _d(u0), _d(tg), float(drop),
                                              int(max_steps), _i(steps), _d(fin), _d(force),
                                              _d(U), _d(secs)))
        out = dict(steps=steps, final_res=fin, force=force, seconds=secs)
        if states:
            out["U"] = U
        return out

    def ilu_order(self) -> np.ndarray:
        o = np.zeros(self.n_cells, np.int64)
        self._check(load().bes_ilu_order(self.h, _i(o)))
        return o

    def flux_batch(self, kind: int, UL, UR, nhat, jacobians: bool = False):
        UL = np.ascontiguousarray(UL, dtype=np.float64)
        UR = np.ascontiguousarray(UR, dtype=np.float64)
        nhat = np.ascontiguousarray(nhat, dtype=np.float64)
        n = UL.shape[0]
        F = np.zeros((n, 5))
        JL = np.zeros((n, 5, 5)) if jacobians else None
        JR = np.zeros((n, 5, 5)) if (jacobians and kind == 0) else None
        self._check(load().bes_flux_batch(self.h, int(kind), n, _d(UL), _d(UR), _d(nhat), _d(F),
                                          _d(JL), _d(JR)))
        return (F, JL, JR) if jacobians else F


def _f(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class WarmStart:
    """The learned warm start (bes_mlp_*) on a context's mesh."""

    def __init__(self, ctx: Context, seed: int = 0):
        L = load()
        h = ctypes.c_void_p()
        rc = L.bes_mlp_create(ctx.h, int(seed), ctypes.byref(h))
        if rc != BES_OK:
            raise BesError(rc, "bes_mlp_create failed")
        self.h = h
        self.n_cells = ctx.n_cells
        n = ctypes.c_int64()
        L.bes_mlp_params(self.h, None, None, ctypes.byref(n))
        self.n_params = n.value

    def _check(self, rc):
        if rc != BES_OK:
            raise BesError(rc, load().bes_mlp_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            load().bes_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.zeros(self.n_params, np.float32)
        self._check(load().bes_mlp_params(self.h, _f(p), None, None))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._check(load().bes_mlp_params(self.h, None, _f(p), None))

    def features(self) -> np.ndarray:
        x = np.zeros((self.n_cells, 3), np.float32)
        self._check(load().bes_mlp_features(self.h, _f(x)))
        return x

    def loss_grad(self, cells, cond, targets):
        cells = np.ascontiguousarray(cells, dtype=np.int64)
        cond = np.ascontiguousarray(cond, dtype=np.float64)
        targets = np.ascontiguousarray(targets, dtype=np.float64)
        n = cells.shape[0]
        loss = ctypes.c_double()
        g = np.zeros(self.n_params, np.float32)
        out = np.zeros((n, 5))
        self._check(load().bes_mlp_loss_grad(self.h, n, _i(cells), _d(cond), _d(targets),
                                             ctypes.byref(loss), _f(g), _d(out)))
        return loss.value, g, out

    def apply_grad(self, grad, lr: float, weight_decay: float):
        g = np.ascontiguousarray(grad, dtype=np.float32)
        self._check(load().bes_mlp_apply_grad(self.h, _f(g), float(lr), float(weight_decay)))

    def train(self, machs, states, steps: int, batch: int = 8192, lr: float = 1e-3,
              weight_decay: float = 1e-4, seed: int = 0):
        machs = np.ascontiguousarray(machs, dtype=np.float64).reshape(-1, 3)
        states = np.ascontiguousarray(states, dtype=np.float64)
        loss = np.zeros(steps)
        self._check(load().bes_mlp_train(self.h, machs.shape[0], _d(machs), _d(states), int(steps),
                                         int(batch), float(lr), float(weight_decay), int(seed),
                                         _d(loss)))
        return loss

    def infer(self, machs) -> np.ndarray:
        machs = np.ascontiguousarray(machs, dtype=np.float64).reshape(-1, 3)
        U = np.zeros((machs.shape[0], self.n_cells, 5))
        self._check(load().bes_mlp_infer(self.h, machs.shape[0], _d(machs), _d(U)))
        return U

    def init_state(self, ctx: Context) -> np.ndarray:
        used = np.zeros(ctx.n_cond, np.int32)
        self._check(load().bes_mlp_init_state(self.h, ctx.h,
                                              used.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
        return used

    def normalisation(self) -> dict:
        out = np.zeros(11)
        self._check(load().bes_mlp_normalisation(self.h, _d(out)))
        return dict(cond_mean=out[:3], cond_std=out[3:6], out_scale=out[6:])
