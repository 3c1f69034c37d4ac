"""Output files and the solve loop against the reference's own files.

The fixtures hold the text the reference wrote (Solver::writeToFile_ after the last step of a
short run, and the residual lines its timeStep_ logged) together with its final state.
CPU tests: the library's writers (bes_write_host) fed with the reference's final state must
reproduce the files.  GPU tests: bes_solve runs the same case from the freestream state and
writes residual.csv and the files, which must match within the 6 printed digits.
"""
import os
import re

import numpy as np
import pytest

from bes_gb300 import lib
from tests import _golden as G
from tests._gpu import context

OUTPUT_CASES = ["output_explicit_vtk", "output_explicit_csv", "output_implicit_vtk",
                "output_explicit2d_vtk", "output_explicit2d_csv"]
NUM = re.compile(r"^[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?$")


def _split(text):
    return [re.split(r"[ ,]", line) for line in text.rstrip("\n").split("\n")]


def compare_text(got, want, rel=0.0, floor=0.0):
    """Token-by-token comparison of two output files.  Non-numeric tokens and the line
    structure must be identical; numbers must agree within `rel` (relative) or `floor`
    (absolute).  Returns the number of numeric tokens whose text differs."""
    a, b = _split(got), _split(want)
    assert len(a) == len(b), (len(a), len(b))
    ndiff = 0
    for la, lb in zip(a, b):
        assert len(la) == len(lb), (la, lb)
        for ta, tb in zip(la, lb):
            if ta == tb:
                continue
            assert NUM.match(ta) and NUM.match(tb), (ta, tb)
            x, y = float(ta), float(tb)
            assert abs(x - y) <= max(rel * abs(y), floor), (ta, tb)
            ndiff += 1
    return ndiff


def _options(info, **extra):
    m = info["meta"]
    kw = dict(solver_type=0 if m["solver"] == "EXPLICIT" else 1,
              local_time_step=1 if m["local"] == "YES" else 0, courant_num=float(m["cfl"]),
              freestream_mach=tuple(m["mach"]), number_of_time_step=int(info["steps"]))
    if m["solver"] == "IMPLICIT":
        kw.update(adaptive_courant_num_max=float(m["cfl_max"]),
                  linear_solver=1 if m["smoother"] == "ILU0" else 0,
                  linear_solver_tol=float(m["lin_tol"]),
                  linear_solver_max_iter=int(m["lin_maxiter"]))
    kw.update(extra)
    return lib.default_options(**kw)


@pytest.mark.parametrize("case", OUTPUT_CASES)
def test_host_writer_reproduces_reference_files(case, tmp_path):
    data, info = G.load(case)
    mesh = G.mesh_of(info)
    opts = _options(info)
    fmt = info["meta"]["out_format"]
    path = str(tmp_path / f"solution_{info['steps']}.{fmt.lower()}")
    lib.write_host(mesh, opts, data["final_state"].reshape(-1, 5), path,
                   lib.OUTPUT_VTK if fmt == "VTK" else lib.OUTPUT_CSV)
    want = str(data["solution"]).replace("{OUT}", str(tmp_path))
    # same input state and the reference's arithmetic: at most a last-digit rounding flip
    assert compare_text(open(path).read(), want, rel=2e-6) <= 2
    if "slip_wall" in data:
        sw = str(tmp_path / "slip.csv")
        lib.write_host(mesh, opts, data["final_state"].reshape(-1, 5), sw,
                       lib.OUTPUT_SLIP_WALL_CSV)
        assert compare_text(open(sw).read(), str(data["slip_wall"]), rel=2e-6) <= 2


def test_output_keys_from_besi(tmp_path):
    p = tmp_path / "case.besi"
    p.write_text("OUTPUT_FOLDER = out dir // comment\nOUTPUT_FORMAT = CSV\n"
                 "OUTPUT_SLIP_WALL = YES\nSAVE_INTERVAL = 25\nCOURANT_NUM = 1.0\n")
    o = lib.output_from_besi(str(p))
    # the reference removes every blank from a value (ReadFile::trimWhiteSpace)
    assert o.folder == b"outdir" and o.format == lib.OUTPUT_CSV
    assert o.slip_wall == 1 and o.save_interval == 25
    d = lib.default_output()
    assert d.folder == b"." and d.format == lib.OUTPUT_VTK and d.slip_wall == 0
    p.write_text("OUTPUT_FORMAT = HDF5\n")
    with pytest.raises(lib.BesError, match="Output format not supported"):
        lib.output_from_besi(str(p))


def test_writer_rejects_unwritable_path(tmp_path):
    data, info = G.load("output_explicit_csv")
    mesh = G.mesh_of(info)
    with pytest.raises(lib.BesError, match="cannot open"):
        lib.write_host(mesh, _options(info), data["final_state"].reshape(-1, 5),
                       str(tmp_path / "missing" / "x.csv"), lib.OUTPUT_CSV)


def _residual_rows(text, strip_step):
    rows = []
    for line in text.rstrip("\n").split("\n"):
        toks = [t for t in line.split(",") if t]
        if strip_step:
            toks = toks[1:]
        rows.append([float(t) for t in toks])
    return np.array(rows)


@pytest.mark.gpu
@pytest.mark.parametrize("case", OUTPUT_CASES)
def test_solve_writes_reference_files(case, tmp_path):
    data, info = G.load(case)
    mesh = G.mesh_of(info)
    m = info["meta"]
    steps = int(info["steps"])
    ctx = lib.Context(mesh, _options(info))
    ctx.set_freestream_state()
    out = lib.default_output(folder=str(tmp_path), format=lib.OUTPUT_VTK if m["out_format"] == "VTK"
                             else lib.OUTPUT_CSV, slip_wall=int(m["out_slip"] == "YES"))
    ctx.solve(out)
    # residual.csv: "<step>," + the reference's timeStep_ line
    res = open(tmp_path / "residual.csv").read()
    steps_col = [int(line.split(",")[0]) for line in res.strip().split("\n")]
    assert steps_col == list(range(1, steps + 1))
    got = _residual_rows(res, True)
    want = _residual_rows(str(data["residual"]), False)
    assert got.shape == want.shape
    scale = np.maximum(np.abs(want[:, :5]), 1e-4 * np.abs(want[:, :5]).max(axis=1, keepdims=True))
    assert np.max(np.abs(got[:, :5] - want[:, :5]) / scale) <= 1e-5
    if m["solver"] == "IMPLICIT":
        assert np.array_equal(got[:, 5], want[:, 5])  # linear iterations
        assert np.allclose(got[:, 6], want[:, 6], rtol=1e-4)  # linear error
    ext = m["out_format"].lower()
    sol = open(tmp_path / f"solution_{steps}.{ext}").read()
    want_sol = str(data["solution"]).replace("{OUT}", str(tmp_path))
    compare_text(sol, want_sol, rel=1e-5, floor=1e-12)
    if m["out_slip"] == "YES":
        compare_text(open(tmp_path / f"slip_wall_{steps}.csv").read(), str(data["slip_wall"]),
                     rel=1e-5, floor=1e-12)
    ctx.close()


@pytest.mark.gpu
def test_solve_save_interval(tmp_path):
    data, info = G.load("output_explicit_vtk")
    mesh = G.mesh_of(info)
    ctx = context(mesh, solver_type=0, local_time_step=1, courant_num=0.8,
                  freestream_mach=(0.7, 0.05, 0.0), number_of_time_step=7)
    ctx.set_freestream_state()
    ctx.solve(lib.default_output(folder=str(tmp_path), save_interval=3, slip_wall=1))
    # files after steps k with k % 3 == 0 (0-based) and after the last one
    names = sorted(os.listdir(tmp_path))
    assert [n for n in names if n.startswith("solution_")] == [
        "solution_1.vtk", "solution_4.vtk", "solution_7.vtk"]
    assert [n for n in names if n.startswith("slip_wall_")] == [
        "slip_wall_1.csv", "slip_wall_4.csv", "slip_wall_7.csv"]
    assert len(open(tmp_path / "residual.csv").read().strip().split("\n")) == 7
    ctx.close()
