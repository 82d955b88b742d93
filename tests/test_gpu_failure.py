"""Failure detection without a GPU fault: a bounded mbarrier wait that nothing arrives on gives up
after its poll limit, sets the context's status word and returns; sei_sync then reports
SEI_ERR_TIMEOUT once, clears the word, and the context keeps working (a step of kernel 'all'
afterwards matches the FP64 oracle).  The same probe with its arrival reports SEI_OK."""
import numpy as np
import pytest

from oracle import oracle_py
from tests.helpers import rel_l2_per_quantity, seeded_dofs

pytestmark = pytest.mark.gpu

SEI_OK, SEI_ERR_TIMEOUT = 0, -4


def test_bounded_wait_gives_up_and_context_stays_usable(built_lib):
    from seissol_gb300 import Context
    from seissol_gb300.lib import SeiError
    ctx = Context(4, device=0, precision=1)
    n = ctx.build_periodic_cube(4, 4, 4, perturb=0.1, seed=2)
    q0 = seeded_dofs(n, 4, 2)
    ctx.set_dofs(q0)
    assert ctx.lib.sei_check_wait_timeout(ctx.h, 4096, 1) == SEI_OK
    assert ctx.lib.sei_sync(ctx.h) == SEI_OK
    assert ctx.lib.sei_check_wait_timeout(ctx.h, 4096, 0) == SEI_OK  # enqueued; the wait runs out
    assert ctx.lib.sei_sync(ctx.h) == SEI_ERR_TIMEOUT
    assert b"gave up" in ctx.lib.sei_last_error(ctx.h)
    assert ctx.lib.sei_sync(ctx.h) == SEI_OK  # reported once
    cells = ctx.get_cells()
    dt = ctx.cfl_timestep(0.5)
    ctx.run("all", dt, 1)
    ctx.sync()
    ref = oracle_py.Oracle(4).steps(q0, cells["star"].astype(np.float64), cells["AplusT"].astype(np.float64),
                                    cells["AminusT"].astype(np.float64), cells["neighbor"], cells["side"],
                                    cells["orient"], dt, 1, cells["face_type"])
    assert max(rel_l2_per_quantity(ctx.get_dofs(), ref)) < 1e-5
    with pytest.raises(SeiError):
        ctx._check(ctx.lib.sei_check_wait_timeout(ctx.h, 0, 0), "sei_check_wait_timeout")
    ctx.close()
