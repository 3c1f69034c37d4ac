"""Checkpoint and resume (bes_checkpoint_save / bes_checkpoint_load): a context resumed from a
checkpoint continues bit for bit as the saved one, explicit (with a freestream ramp still
running, so the step counter matters) and implicit (a batch with adaptive CFL, one condition
frozen); a mismatched context refuses the file."""
import numpy as np
import pytest

from bes_gb300 import build as nbuild
from bes_gb300 import lib, meshgen

pytestmark = pytest.mark.gpu

MACHS = [(0.5, 0.0, 0.0), (0.7, 0.05, 0.0), meshgen.freestream_mach_vector(0.6, 3.0, -2.0)]


def test_explicit_resume_is_bitwise(tmp_path):
    nbuild.build()
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    o = lib.default_options(solver_type=0, local_time_step=1, courant_num=0.8,
                            freestream_mach=(0.6, 0.0, 0.0), freestream_ramp=8,
                            freestream_ramp_start_frac=0.4)
    a = lib.Context(mesh, o)
    ha = a.explicit_iterations(12)
    b = lib.Context(mesh, o)
    b.explicit_iterations(5)
    path = str(tmp_path / "explicit.ckpt")
    b.checkpoint_save(path)
    b.close()
    c = lib.Context(mesh, o)
    c.checkpoint_load(path)
    hc = c.explicit_iterations(7)
    assert np.array_equal(hc, ha[5:])
    assert np.array_equal(c.get_state(), a.get_state())
    a.close()
    c.close()


@pytest.mark.parametrize("precision", [0, 2])
def test_implicit_batch_resume_is_bitwise(tmp_path, precision):
    nbuild.build()
    mesh = meshgen.bump_channel(12, 4, 4, 0.08)
    o = lib.default_options(solver_type=1, local_time_step=1, courant_num=10.0,
                            adaptive_courant_num_max=500.0, linear_solver=1,
                            linear_solver_tol=1e-2, linear_solver_max_iter=200,
                            precision=precision)
    a = lib.Context(mesh, o, machs=MACHS)
    a.implicit_steps(3)
    a.set_active([1, 0, 1])
    ha = a.implicit_steps(4)
    b = lib.Context(mesh, o, machs=MACHS)
    b.implicit_steps(3)
    b.set_active([1, 0, 1])
    b.implicit_steps(1)
    path = str(tmp_path / "implicit.ckpt")
    b.checkpoint_save(path)
    b.close()
    c = lib.Context(mesh, o, machs=MACHS)
    c.checkpoint_load(path)
    hc = c.implicit_steps(3)
    assert np.array_equal(hc, ha[1:])
    assert np.array_equal(c.get_state(), a.get_state())
    a.close()
    c.close()
    # another condition count (or solver type, or mesh) refuses the file
    d = lib.Context(mesh, o, machs=MACHS[:2])
    with pytest.raises(lib.BesError) as e:
        d.checkpoint_load(path)
    assert e.value.code == 1
    d.close()
