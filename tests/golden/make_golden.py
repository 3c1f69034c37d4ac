"""Regenerate the golden fixtures in this folder from the reference itself.

Runs the patched reference build (oracle/ref, compiled from the reference sources into
oracle/_ref/) on small generated meshes at OMP_NUM_THREADS=1 and stores its FP64 binary dumps
as compressed .npz fixtures.  Only this script reads the reference; the fixtures are what
the tests use (the reference is not available where the GPU tests run).

    python tests/golden/make_golden.py --ref /path/to/reference

The reference checkout may also be given as the environment variable BES_REFERENCE_DIR.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from bes_gb300 import meshgen  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "bes_ref_harness")

# name -> (mesh builder, options, steps, mode, dump_ops)
CASES = {
    "explicit_bump_local": (lambda: meshgen.bump_channel(12, 4, 4, 0.04),
                            dict(solver="EXPLICIT", local="YES", cfl=0.8, mach=(0.5, 0, 0)),
                            50, "explicit", True),
    "explicit_bump_global": (lambda: meshgen.bump_channel(12, 4, 4, 0.04),
                             dict(solver="EXPLICIT", local="NO", cfl=0.8, mach=(0.5, 0, 0)),
                             20, "explicit", False),
    "explicit_gauss_pitch": (lambda: meshgen.gaussian_box(8, 4, 8),
                             dict(solver="EXPLICIT", local="YES", cfl=0.8,
                                  mach=meshgen.freestream_mach_vector(0.7, 3.0, -2.0)),
                             20, "explicit", True),
    "explicit_bump_supersonic": (lambda: meshgen.bump_channel(12, 4, 4, 0.08),
                                 dict(solver="EXPLICIT", local="YES", cfl=0.8,
                                      mach=(1.6, 0, 0)),
                                 20, "explicit", True),
    "explicit_bump_ramp": (lambda: meshgen.bump_channel(12, 4, 4, 0.08),
                           dict(solver="EXPLICIT", local="YES", cfl=0.8, mach=(0.7, 0, 0),
                                fs_ramp=8, fs_frac=0.3),
                           15, "explicit", False),
    "implicit_bump_jacobi": (lambda: meshgen.bump_channel(12, 4, 4, 0.08),
                             dict(solver="IMPLICIT", local="YES", cfl=10.0, cfl_max=1000.0,
                                  mach=(0.84, 0, 0), smoother="DAMPED_JACOBI", lin_tol=1e-2,
                                  lin_maxiter=300),
                             12, "implicit", True),
    # 2-D (triangles, 4 conserved variables; fixtures in the 3-D layout, see the harness).
    # The implicit case's 4x4-block systems go through the linear-solver facade as 5x5 blocks
    # with a decoupled spanwise-momentum row (oracle/ref/stubs/amgcl/facade.hpp).
    "explicit_bump2d_local": (lambda: meshgen.bump_channel_2d(24, 8, 0.08),
                              dict(solver="EXPLICIT", local="YES", cfl=0.8, mach=(0.6, 0.04, 0)),
                              50, "explicit", "geometry"),
    "implicit_bump2d_ilu0": (lambda: meshgen.bump_channel_2d(24, 8, 0.08),
                             dict(solver="IMPLICIT", local="YES", cfl=10.0, cfl_max=1000.0,
                                  mach=(0.6, 0.04, 0), smoother="ILU0", lin_tol=1e-2,
                                  lin_maxiter=300),
                             12, "implicit", False),
    "implicit_bump_ilu0": (lambda: meshgen.bump_channel(12, 4, 4, 0.08),
                           dict(solver="IMPLICIT", local="YES", cfl=10.0, cfl_max=1000.0,
                                mach=(0.84, 0, 0), smoother="ILU0", lin_tol=1e-2,
                                lin_maxiter=300),
                           12, "implicit", True),
    # implicit with a global time step, and on the pitched Gaussian box (histories only)
    "implicit_bump_global": (lambda: meshgen.bump_channel(12, 4, 4, 0.08),
                             dict(solver="IMPLICIT", local="NO", cfl=10.0, cfl_max=1000.0,
                                  mach=(0.84, 0, 0), smoother="DAMPED_JACOBI", lin_tol=1e-2,
                                  lin_maxiter=300),
                             8, "implicit", False),
    "implicit_gauss_pitch": (lambda: meshgen.gaussian_box(8, 4, 8),
                             dict(solver="IMPLICIT", local="YES", cfl=10.0, cfl_max=1000.0,
                                  mach=meshgen.freestream_mach_vector(0.7, 3.0, -2.0),
                                  smoother="ILU0", lin_tol=1e-2, lin_maxiter=300),
                             8, "implicit", False),
    "implicit_bump_ramp": (lambda: meshgen.bump_channel(12, 4, 4, 0.08),
                           dict(solver="IMPLICIT", local="YES", cfl=10.0, cfl_max=1000.0,
                                mach=(0.7, 0, 0), smoother="ILU0", lin_tol=1e-2,
                                lin_maxiter=300, fs_ramp=5, fs_frac=0.3),
                           8, "implicit", False),
    "implicit_bump2d_jacobi_global": (lambda: meshgen.bump_channel_2d(24, 8, 0.08),
                                      dict(solver="IMPLICIT", local="NO", cfl=10.0,
                                           cfl_max=1000.0, mach=(0.6, 0.04, 0),
                                           smoother="DAMPED_JACOBI", lin_tol=1e-2,
                                           lin_maxiter=300),
                                      8, "implicit", False),
    # the reference's own converged state: a 4 % bump at Mach 0.5 solved by its implicit solver
    # (adaptive CFL 10 -> 1000) for 200 steps, where its residual has fallen to the rounding
    # floor (about 4e-12 of the first)
    "implicit_bump_converged": (lambda: meshgen.bump_channel(24, 8, 6, 0.04),
                                dict(solver="IMPLICIT", local="YES", cfl=10.0, cfl_max=1000.0,
                                     mach=(0.5, 0, 0), smoother="ILU0", lin_tol=1e-2,
                                     lin_maxiter=300),
                                200, "implicit", False),
    # the rest of the option surface on the path: `besi` lines added to the case file, `oracle`
    # the matching keyword arguments of the CPU restatement
    "explicit_bump_options": (lambda: meshgen.bump_channel(12, 4, 4, 0.08),
                              dict(solver="EXPLICIT", local="YES", cfl=0.8, mach=(0.7, 0.05, 0),
                                   besi=["MULTI_TIME_STEP_OPTIONS = 3, 0.1, 0.5, 1.0",
                                         "VENKATAKRISHNAN_FACTOR = 2.0",
                                         "HARTEN_CORRECTION_LIMIT = 0.2",
                                         "SPECIFIC_HEAT_RATIO = 1.3", "GAS_CONSTANT = 300.0"],
                                   oracle=dict(alpha=(0.1, 0.5, 1.0), venkat_k=2.0, harten=0.2,
                                               gamma=1.3, gas_constant=300.0)),
                              20, "explicit", False),
    "implicit_bump_options": (lambda: meshgen.bump_channel(12, 4, 4, 0.08),
                              dict(solver="IMPLICIT", local="YES", cfl=10.0, cfl_max=1000.0,
                                   mach=(0.7, 0.05, 0), smoother="ILU0", lin_tol=1e-2,
                                   lin_maxiter=300, cfl_exp=(0.5, 2.0),
                                   besi=["SPECIFIC_HEAT_RATIO = 1.3",
                                         "VENKATAKRISHNAN_FACTOR = 2.0"],
                                   oracle=dict(gamma=1.3, venkat_k=2.0)),
                              8, "implicit", False),
}

# the reference's own output files (Solver::writeToFile_ after the last step, and the residual
# lines its timeStep_ appends): name -> (mesh builder, options, steps, mode)
OUTPUT_CASES = {
    "output_explicit_vtk": (lambda: meshgen.bump_channel(12, 4, 4, 0.08),
                            dict(solver="EXPLICIT", local="YES", cfl=0.8, mach=(0.7, 0.05, 0),
                                 out_format="VTK", out_slip="YES"),
                            6, "explicit"),
    "output_explicit_csv": (lambda: meshgen.gaussian_box(8, 4, 8),
                            dict(solver="EXPLICIT", local="YES", cfl=0.8,
                                 mach=meshgen.freestream_mach_vector(0.6, 2.0, -1.0),
                                 out_format="CSV", out_slip="NO"),
                            4, "explicit"),
    "output_explicit2d_vtk": (lambda: meshgen.bump_channel_2d(24, 8, 0.08),
                              dict(solver="EXPLICIT", local="YES", cfl=0.8, mach=(0.6, 0.04, 0),
                                   out_format="VTK", out_slip="YES"),
                              6, "explicit"),
    "output_explicit2d_csv": (lambda: meshgen.bump_channel_2d(24, 8, 0.08),
                              dict(solver="EXPLICIT", local="NO", cfl=0.8, mach=(0.6, 0.04, 0),
                                   out_format="CSV", out_slip="NO"),
                              4, "explicit"),
    "output_implicit_vtk": (lambda: meshgen.bump_channel(12, 4, 4, 0.08),
                            dict(solver="IMPLICIT", local="YES", cfl=10.0, cfl_max=1000.0,
                                 mach=(0.84, 0, 0), smoother="DAMPED_JACOBI", lin_tol=1e-2,
                                 lin_maxiter=300, out_format="VTK", out_slip="YES"),
                            4, "implicit"),
}

KAT_MACHS = {"kat_subsonic": (0.5, 0.1, -0.05), "kat_supersonic": (2.0, 0.2, 0.1)}


def besi_text(mesh_path: str, out_dir: str, o: dict, steps: int) -> str:
    lines = [
        "MESH_FORMAT = GMSH",
        f"MESH_FILE = {mesh_path}",
        f"OUTPUT_FOLDER = {out_dir}",
        f"SOLVER_TYPE = {o['solver']}",
        f"LOCAL_TIME_STEP = {o['local']}",
        f"COURANT_NUM = {o['cfl']!r}",
        f"NUMBER_OF_TIME_STEP = {steps}",
        "SAVE_INTERVAL = 100000",
        "FREESTREAM_MACH = " + ", ".join(repr(float(x)) for x in o["mach"]),
    ]
    if o.get("out_format"):
        lines += [f"OUTPUT_FORMAT = {o['out_format']}", f"OUTPUT_SLIP_WALL = {o['out_slip']}"]
    if o.get("fs_ramp"):
        lines += [f"FREESTREAM_RAMP = {o['fs_ramp']}",
                  f"FREESTREAM_RAMP_START_FRAC = {o['fs_frac']!r}"]
    if o["solver"] == "IMPLICIT":
        e0, e1 = o.get("cfl_exp", (1.0, 1.0))
        lines += [
            f"ADAPTIVE_COURANT_NUM_MAX = {o['cfl_max']!r}",
            f"ADAPTIVE_COURANT_NUM_EXPONENT = {e0!r}, {e1!r}",
            "LINEAR_SOLVER = GMRES",
            "AMG_PRECOND_COARSENER = AGGREGATION",
            f"AMG_PRECOND_SMOOTHER = {o['smoother']}",
            f"LINEAR_SOLVER_MAX_ITER = {o['lin_maxiter']}",
            f"LINEAR_SOLVER_ABS_TOL = {o['lin_tol']!r}",
        ]
    lines += o.get("besi", [])
    return "\n".join(lines) + "\n"


def _load(d, name, dtype=np.float64):
    p = os.path.join(d, name)
    return np.fromfile(p, dtype=dtype) if os.path.exists(p) else None


def run_case(name, builder, opts, steps, mode, dump):
    mesh = builder()
    with tempfile.TemporaryDirectory() as tmp:
        msh = os.path.join(tmp, "mesh.msh")
        meshgen.write_gmsh(mesh, msh)
        besi = os.path.join(tmp, "case.besi")
        with open(besi, "w") as f:
            f.write(besi_text(msh, tmp, opts, steps))
        extra = ["dump_ops"] if dump is True else ([dump] if dump else [])
        args = [HARNESS, besi, tmp, str(steps), mode] + extra
        env = dict(os.environ, OMP_NUM_THREADS="1")
        subprocess.run(args, check=True, env=env, stdout=subprocess.DEVNULL)
        out = {"n_cells": mesh.n_cells}
        for key in ("residual_history", "implicit_history", "final_state", "op_state", "op_dt",
                    "op_grad", "op_limiter", "op_face_UL", "op_face_UR", "op_face_flux",
                    "op_rhs", "op_mat_val", "geo_volume", "geo_centroid", "geo_vec_to_face",
                    "geo_weight", "geo_face_S", "geo_face_n", "geo_face_area", "geo_face_center"):
            a = _load(tmp, key + ".bin")
            if a is not None:
                out[key] = a
        for key in ("geo_cell_face", "geo_cell_adj", "geo_face_owner", "geo_face_neigh",
                    "geo_face_type", "geo_muscl_slot", "op_mat_rowptr", "op_mat_col"):
            a = _load(tmp, key + ".bin", np.int64)
            if a is not None:
                out[key] = a
    meta = dict(opts)
    meta["mach"] = list(map(float, opts["mach"]))
    out["meta"] = np.array(repr(dict(meta=meta, steps=steps, mode=mode, mesh=mesh.name)))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(f"{name}: {mesh.n_cells} cells, {len(out)} arrays")


def run_output_case(name, builder, opts, steps, mode):
    """Fixture of the reference's output files; the output folder in the VTK title line is
    replaced by {OUT}."""
    mesh = builder()
    with tempfile.TemporaryDirectory() as tmp:
        msh = os.path.join(tmp, "mesh.msh")
        meshgen.write_gmsh(mesh, msh)
        besi = os.path.join(tmp, "case.besi")
        with open(besi, "w") as f:
            f.write(besi_text(msh, tmp, opts, steps))
        subprocess.run([HARNESS, besi, tmp, str(steps), mode, "write"], check=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"), stdout=subprocess.DEVNULL)
        out = {"n_cells": mesh.n_cells, "final_state": _load(tmp, "final_state.bin")}
        ext = opts["out_format"].lower()
        files = {"solution": f"solution_{steps}.{ext}", "residual": "ref_residual.csv"}
        if opts["out_slip"] == "YES":
            files["slip_wall"] = f"slip_wall_{steps}.csv"
        for key, fn in files.items():
            with open(os.path.join(tmp, fn)) as f:
                out[key] = np.array(f.read().replace(tmp, "{OUT}"))
    meta = dict(opts)
    meta["mach"] = list(map(float, opts["mach"]))
    out["meta"] = np.array(repr(dict(meta=meta, steps=steps, mode=mode, mesh=mesh.name)))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(f"{name}: {mesh.n_cells} cells, files {sorted(files)}")


def run_kat(name, mach, n=96, seed=7):
    rng = np.random.default_rng(seed)
    rho = rng.uniform(0.5, 2.0, (n, 2))
    vel = rng.uniform(-1.2, 1.2, (n, 2, 3))
    p = rng.uniform(0.3, 1.5, (n, 2))
    gamma = 1.4
    U = np.zeros((n, 2, 5))
    U[..., 0] = rho
    U[..., 1:4] = rho[..., None] * vel
    U[..., 4] = p / (gamma - 1.0) + 0.5 * rho * (vel ** 2).sum(-1)
    nh = rng.normal(size=(n, 3))
    nh /= np.linalg.norm(nh, axis=1, keepdims=True)
    rec = np.concatenate([U[:, 0], U[:, 1], nh], axis=1)
    mesh = meshgen.bump_channel(6, 2, 2, 0.04)
    with tempfile.TemporaryDirectory() as tmp:
        msh = os.path.join(tmp, "mesh.msh")
        meshgen.write_gmsh(mesh, msh)
        besi = os.path.join(tmp, "case.besi")
        with open(besi, "w") as f:
            f.write(besi_text(msh, tmp, dict(solver="EXPLICIT", local="YES", cfl=0.8, mach=mach), 1))
        rec.tofile(os.path.join(tmp, "kat_in.bin"))
        subprocess.run([HARNESS, besi, tmp, str(n), "kat"], check=True,
                       stdout=subprocess.DEVNULL, env=dict(os.environ, OMP_NUM_THREADS="1"))
        out = np.fromfile(os.path.join(tmp, "kat_out.bin")).reshape(n, -1)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), inputs=rec, outputs=out,
                        mach=np.array(mach, dtype=np.float64))
    print(f"{name}: {n} records")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("BES_REFERENCE_DIR"))
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    if not a.ref:
        sys.exit("give the reference checkout with --ref or BES_REFERENCE_DIR")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={a.ref}", "-j8"],
                   check=True, stdout=subprocess.DEVNULL)
    if not os.path.exists(HARNESS):
        sys.exit("reference harness did not build")
    for name, (b, o, s, m, d) in CASES.items():
        if a.only and a.only != name:
            continue
        run_case(name, b, o, s, m, d)
    for name, (b, o, s, m) in OUTPUT_CASES.items():
        if a.only and a.only != name:
            continue
        run_output_case(name, b, o, s, m)
    for name, mach in KAT_MACHS.items():
        if a.only and a.only != name:
            continue
        run_kat(name, mach)


if __name__ == "__main__":
    main()
