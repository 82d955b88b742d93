"""GPU edge cases of the element update through the C ABI: ragged and minimal meshes (a single
cell, 33 cells: one full block of 32 and one more, a partial tile of the tensor-core kernels),
zero steps, zero data, and rejected inputs.  Tolerances: 1e-5 relative L2 per quantity of the
field against the FP64 oracle after two steps (both paths), exact where the result is exact."""
import numpy as np
import pytest

from oracle import oracle_py
from tests.helpers import rel_l2_per_quantity, seeded_dofs

pytestmark = pytest.mark.gpu

PREC_F16X3 = 1


def _cut(order, keep, seed):
    """The first `keep` cells of a periodic 4x4x4 cube, faces towards dropped cells made outflow."""
    from seissol_gb300 import Context
    base = Context(order, device=0)
    base.build_periodic_cube(4, 4, 4, perturb=0.05, seed=seed)
    cells = base.get_cells()
    dt = base.cfl_timestep(0.5)
    base.close()
    cut = {k: np.ascontiguousarray(v[:keep]) for k, v in cells.items()}
    ft = np.array(cut["face_type"], dtype=np.int8)
    nb = np.array(cut["neighbor"])
    ft[nb >= keep] = 2
    nb[nb >= keep] = 0
    return cut, nb, ft, dt


@pytest.mark.parametrize("precision", [0, PREC_F16X3])
@pytest.mark.parametrize("keep", [1, 33])
@pytest.mark.parametrize("order", [4, 6])
def test_ragged_meshes_two_steps(built_lib, order, keep, precision):
    from seissol_gb300 import Context
    cut, nb, ft, dt = _cut(order, keep, 31)
    q0 = seeded_dofs(keep, order, 31)
    ctx = Context(order, device=0, precision=precision)
    ctx.set_cells(cut["star"], cut["AplusT"], cut["AminusT"], nb, cut["side"], cut["orient"], ft)
    ctx.set_dofs(q0)
    ctx.run("all", dt, 2)
    ctx.sync()
    got = ctx.get_dofs()
    ctx.close()
    ref = oracle_py.Oracle(order).steps(q0, cut["star"].astype(np.float64), cut["AplusT"].astype(np.float64),
                                        cut["AminusT"].astype(np.float64), nb, cut["side"], cut["orient"], dt, 2, ft)
    errs = rel_l2_per_quantity(got, ref)
    assert max(errs) < 1e-5, errs


@pytest.mark.parametrize("precision", [0, PREC_F16X3])
def test_zero_steps_and_zero_data(built_lib, precision):
    """Zero steps leave the DOFs as they are, bit for bit; a zero field stays exactly zero."""
    from seissol_gb300 import Context
    ctx = Context(4, device=0, precision=precision)
    n = ctx.build_periodic_cube(4, 4, 4, perturb=0.05, seed=5)
    dt = ctx.cfl_timestep(0.5)
    q0 = seeded_dofs(n, 4, 5)
    ctx.set_dofs(q0)
    ctx.run("all", dt, 0)
    ctx.sync()
    assert np.array_equal(ctx.get_dofs(), q0)
    ctx.set_dofs(np.zeros_like(q0))
    ctx.run("all", dt, 3)
    ctx.sync()
    assert not ctx.get_dofs().any()
    ctx.close()


def test_rejected_inputs(built_lib):
    """A non-finite operator entry, a non-finite or negative time step and a negative step count
    are errors (SEI_ERR_NAN, SEI_ERR_ARG), not silent results; a rejected call changes nothing, so
    the context keeps its mesh and stays usable."""
    from seissol_gb300 import Context, SeiError
    ctx = Context(4, device=0)
    n = ctx.build_periodic_cube(4, 4, 4, perturb=0.0, seed=7)
    cells = ctx.get_cells()
    star = np.array(cells["star"])
    star[2, 1, 6] = np.inf  # entry (q 6, p 0) of a star matrix, one of its structural non-zeros
    with pytest.raises(SeiError, match="SEI_ERR_NAN"):
        ctx.set_cells(star, cells["AplusT"], cells["AminusT"], cells["neighbor"], cells["side"], cells["orient"],
                      cells["face_type"])
    for dt, steps in ((float("nan"), 1), (-1e-4, 1), (1e-4, -1)):
        with pytest.raises(SeiError, match="SEI_ERR_ARG"):
            ctx.run("all", dt, steps)
    q0 = seeded_dofs(n, 4, 7)
    ctx.set_dofs(q0)
    ctx.run("all", ctx.cfl_timestep(0.5), 1)
    ctx.sync()
    assert np.isfinite(ctx.get_dofs()).all()
    ctx.close()
