"""CPU-only checks of the native library: it loads, exports every symbol the C header
declares, its struct mirrors match, and its host-side mesh build and .besi / Gmsh readers agree
with the reference (golden geometry) and with the oracle."""
import os
import re
import tempfile

import numpy as np
import pytest

from bes_gb300 import build as nbuild
from bes_gb300 import lib, meshgen
from tests import _golden as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def native():
    nbuild.build()
    return lib.load()


def declared_functions():
    names = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(bes_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_exports_every_declared_symbol(native):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(native, n), n
    assert set(names) == set(lib.EXPORTED)


def test_struct_mirrors_match(native):
    import ctypes
    out = (ctypes.c_int64 * 3)()
    native.bes_abi_sizes(out)
    assert out[0] == ctypes.sizeof(lib.Options)
    assert out[1] == ctypes.sizeof(lib.MeshArrays)
    assert out[2] == ctypes.sizeof(lib.Output)


def test_build_info_names_sm103a(native):
    assert b"sm_103a" in native.bes_build_info()


@pytest.mark.parametrize("case", G.CASES + G.CASES_2D)
def test_host_geometry_matches_reference(case):
    ref, info = G.load(case)
    if "geo_volume" not in ref:
        pytest.skip("no geometry dump")
    mesh = G.mesh_of(info)
    g = lib.host_geometry(mesh)
    for k in ("volume", "centroid", "face_S", "face_area"):
        np.testing.assert_array_equal(g[k].ravel(), ref["geo_" + k], err_msg=k)
    for k in ("face_owner", "face_neigh", "face_type"):
        np.testing.assert_array_equal(g[k].ravel(), ref["geo_" + k], err_msg=k)
    nfc = mesh.dim + 1  # faces per cell; the fixture pads triangles' fourth slot with -1
    np.testing.assert_array_equal(g["muscl_slot"][:, :nfc],
                                  ref["geo_muscl_slot"].reshape(-1, 4)[:, :nfc])


def test_renumbering_is_a_permutation_and_groups_faces():
    m = meshgen.gaussian_box(10, 6, 10)
    g = lib.host_geometry(m)
    nc, nf = m.n_cells, g["face_area"].shape[0]
    assert np.array_equal(np.sort(g["cell_new2ref"]), np.arange(nc))
    assert np.array_equal(np.sort(g["face_new2ref"]), np.arange(nf))
    kinds = g["face_type"][g["face_new2ref"]]
    # interior faces first, then slip walls, then freestream
    assert np.all(np.diff(kinds) >= 0)


def _pages_per_warp(new2ref, own, nb):
    """Average number of distinct 32-cell pages the face neighbours of a warp of 32
    consecutive cells fall into (the gather footprint of a cell sweep)."""
    n = len(new2ref)
    inv = np.empty_like(new2ref)
    inv[new2ref] = np.arange(n)
    mask = nb >= 0
    a, b = inv[own[mask]], inv[nb[mask]]
    cells = np.concatenate([a, b])
    nbrs = np.concatenate([b, a])
    key = (cells // 32) * (n // 32 + 1) + nbrs // 32
    uniq = np.unique(key)
    return len(uniq) / (n / 32)


def test_renumbering_keeps_neighbours_close():
    """Cells are numbered colour by colour, each colour grouped by its cells' lower-neighbour
    pattern and in reverse Cuthill-McKee order inside a group: the neighbours of a warp of
    consecutive cells stay in far fewer pages than in a random order.  (The pattern groups
    cost some locality, 0.43x of random here against under 0.25x for plain colour-major RCM; the
    block-ILU(0) sweeps gain 22 % from them and the explicit kernels measured unchanged.)"""
    m = meshgen.bump_channel(30, 10, 8, 0.04)
    g = lib.host_geometry(m)
    own, nb = g["face_owner"], g["face_neigh"]
    new = _pages_per_warp(g["cell_new2ref"], own, nb)
    rnd = _pages_per_warp(np.random.default_rng(0).permutation(len(g["cell_new2ref"])), own, nb)
    assert new < 0.5 * rnd


def test_mesh_errors_are_reported():
    m = meshgen.bump_channel(4, 2, 2, 0.04)
    bad = meshgen.TetMesh(m.nodes, m.tets, m.btris[2:], m.btags[2:])
    with pytest.raises(lib.BesError) as e:
        lib.host_geometry(bad)
    assert e.value.code == 4
    bad2 = meshgen.TetMesh(m.nodes, m.tets, m.btris, np.full_like(m.btags, 7))
    with pytest.raises(lib.BesError):
        lib.host_geometry(bad2)


def test_triangle_mesh_errors_are_reported():
    m = meshgen.bump_channel_2d(8, 4, 0.08)
    # an edge with one triangle and no boundary line
    bad = meshgen.TetMesh(m.nodes, m.tets, m.btris[3:], m.btags[3:])
    with pytest.raises(lib.BesError) as e:
        lib.host_geometry(bad)
    assert e.value.code == 4 and "one triangle" in str(e.value)
    # a boundary line with an unknown tag
    with pytest.raises(lib.BesError, match="unknown boundary tag"):
        lib.host_geometry(meshgen.TetMesh(m.nodes, m.tets, m.btris, np.full_like(m.btags, 7)))


def test_gmsh_reader_2d_rules(tmp_path):
    """2-D files (largest physical-name dimension 2): lines are the boundary, triangles the
    cells; a line after a triangle and a tetrahedron are rejected (Mesh::readGmsh reads the
    boundary first and has no 3-D element in a 2-D problem)."""
    m = meshgen.bump_channel_2d(4, 2, 0.08)
    p = str(tmp_path / "m.msh")
    meshgen.write_gmsh(m, p)
    text = open(p).read()
    head, rest = text.split("$Elements\n")
    count, body = rest.split("\n", 1)
    rows = body.split("$EndElements")[0].strip().split("\n")
    nb = m.btris.shape[0]
    # move the first boundary line behind the triangles
    swapped = rows[1:nb] + rows[nb:] + rows[:1]
    q = str(tmp_path / "late_line.msh")
    with open(q, "w") as f:
        f.write(head + "$Elements\n" + count + "\n" + "\n".join(swapped) + "\n$EndElements\n")
    with pytest.raises(lib.BesError, match="boundary line listed after a triangle"):
        lib.read_gmsh(q)
    # a tetrahedron in the 2-D file
    extra = f"{len(rows) + 1} 4 2 3 3 1 2 3 4"
    r = str(tmp_path / "tet.msh")
    with open(r, "w") as f:
        f.write(head + "$Elements\n" + str(len(rows) + 1) + "\n" + "\n".join(rows + [extra])
                + "\n$EndElements\n")
    with pytest.raises(lib.BesError, match="tetrahedron in a 2D problem"):
        lib.read_gmsh(r)


@pytest.mark.parametrize("make", [lambda: meshgen.gaussian_box(6, 4, 6),
                                  lambda: meshgen.bump_channel_2d(12, 4, 0.08)],
                         ids=["tetrahedra", "triangles"])
def test_gmsh_reader_round_trip(make):
    m = make()
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "m.msh")
        meshgen.write_gmsh(m, p)
        r = lib.read_gmsh(p)
    np.testing.assert_array_equal(r.nodes, m.nodes)
    np.testing.assert_array_equal(r.tets, m.tets)
    np.testing.assert_array_equal(r.btris, m.btris)
    np.testing.assert_array_equal(r.btags, m.btags)


def _write(d, text):
    p = os.path.join(d, "case.besi")
    with open(p, "w") as f:
        f.write(text)
    return p


def test_besi_parser_reference_keys_and_defaults():
    with tempfile.TemporaryDirectory() as d:
        p = _write(d, """// comment line
MESH_FORMAT = GMSH
MESH_FILE = mesh dir/mesh.msh // trailing comment
SOLVER_TYPE = IMPLICIT
LOCAL_TIME_STEP = YES
COURANT_NUM = 10
ADAPTIVE_COURANT_NUM_MAX = 1000
ADAPTIVE_COURANT_NUM_EXPONENT = 0.5, 2
MULTI_TIME_STEP_OPTIONS = 3, 0.1, 0.5, 1.0
FREESTREAM_MACH = 0.84, 0.1, 0
LINEAR_SOLVER = FGMRES
AMG_PRECOND_COARSENER = SMOOTHED_AGGREGATION
AMG_PRECOND_SMOOTHER = ILU0
LINEAR_SOLVER_MAX_ITER = 50
LINEAR_SOLVER_ABS_TOL = 1e-2
NUMBER_OF_TIME_STEP = 7
SAVE_INTERVAL = 10
""")
        o, mesh = lib.options_from_besi(p)
    assert mesh == "meshdir/mesh.msh"  # the reference strips every blank
    assert o.solver_type == 1 and o.local_time_step == 1
    assert o.courant_num == 10 and o.adaptive_courant_num_max == 1000
    assert tuple(o.adaptive_courant_num_exponent) == (0.5, 2.0)
    assert o.n_stage == 3 and tuple(o.stage_coeff[:3]) == (0.1, 0.5, 1.0)
    assert tuple(o.freestream_mach) == (0.84, 0.1, 0.0)
    assert o.linear_solver == 1 and o.linear_solver_max_iter == 50
    assert o.linear_solver_tol == 1e-2 and o.number_of_time_step == 7
    # untouched defaults (src/Config.cpp:73-114)
    assert o.venkatakrishnan_factor == 5.0 and o.harten_correction_limit == 0.05
    assert o.gas_constant == 287.0 and o.specific_heat_ratio == 1.4
    assert o.precision == 0
    # 0: each Jacobian block added once per conserved variable of the mesh, as the reference
    assert o.jacobian_repeat == 0


@pytest.mark.parametrize("word,value", [("FP64", 0), ("MIXED", 1), ("MIXED_PACKED", 2)])
def test_besi_precision_key(word, value):
    with tempfile.TemporaryDirectory() as d:
        o, _ = lib.options_from_besi(_write(d, f"PRECISION = {word}\n"))
    assert o.precision == value


@pytest.mark.parametrize("word,value", [("AUTO", 0), ("PER_COLOUR", 1), ("PERSISTENT", 2),
                                        ("PER_COLOUR_LOADS_FIRST", 3)])
def test_besi_sweep_kernel_key(word, value):
    with tempfile.TemporaryDirectory() as d:
        o, _ = lib.options_from_besi(_write(d, f"SWEEP_KERNEL = {word}\n"))
    assert o.sweep_kernel == value


@pytest.mark.parametrize("line", ["NOT_A_KEY = 1", "SOLVER_TYPE = SEMI", "FLUX_SCHEME = AUSM",
                                  "FREESTREAM_MACH = 0.5, 0", "GMRES_RESTART = 33",
                                  "PRECISION = FP16", "SWEEP_KERNEL = EARLY"])
def test_besi_parser_is_strict(line):
    with tempfile.TemporaryDirectory() as d:
        p = _write(d, "MESH_FORMAT = GMSH\n" + line + "\n")
        with pytest.raises(lib.BesError) as e:
            lib.options_from_besi(p)
    assert e.value.code == 5


def test_host_build_is_independent_of_the_thread_count():
    """The host mesh build runs its independent per-cell and per-face loops on several threads;
    one thread gives the same geometry and numbering, and every device-layout array (weights,
    face lists, ELL slots, colouring, both block-ILU(0) schedules) byte for byte
    (BES_HOST_THREADS is read once per process, so each count runs in a process of its own)."""
    import json
    import subprocess
    import sys
    code = ("import json, sys, hashlib; sys.path.insert(0, %r); from bes_gb300 import lib, meshgen; "
            "m = meshgen.gaussian_box(40, 20, 40, 1.05); g = lib.host_geometry(m); "
            "d = {k: hashlib.sha256(v.tobytes()).hexdigest() for k, v in g.items()}; "
            "d['layout'] = lib.host_layout_digest(m); "
            "d['layout_rcm'] = lib.host_layout_digest(m, rcm_ilu_order=True); "
            "d['layout_exact'] = lib.host_layout_digest(m, muscl_exact=True); "
            "print(json.dumps(d))"
            % os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    outs = []
    for n in ("1", "8"):
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                           env=dict(os.environ, BES_HOST_THREADS=n), timeout=300)
        assert r.returncode == 0, r.stderr[-2000:]
        outs.append(json.loads(r.stdout.strip().splitlines()[-1]))
    assert len(outs[0]["layout"]) == 30
    assert outs[0] == outs[1]
