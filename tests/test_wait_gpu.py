"""The bounded waits of the FP32c Coulomb kernels' copy ring.

Every wait on a ring barrier gives up after a %globaltimer limit, raises SG_TIMEOUT in
the context's error word, waits (bounded) for the copies the block has issued and
returns.  sg_set_wait_test makes each block also wait, once its chosen tile has
arrived, on a barrier that nothing arrives at, so the limit runs out while every real
copy still lands: the test exercises the timeout path without leaving a copy in flight.
The attempt must then be refused (no accepted step from incomplete sums), the call must
return SG_TIMEOUT, and after a new upload the same context must integrate the cloud
exactly as a fresh run does."""
import numpy as np
import pytest

from simbuca_gb300 import abi, configs
from simbuca_gb300.abi import SG_PREC_FP32C
from simbuca_gb300.api import Batch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("variant", [-1, 9])
def test_ring_wait_times_out_and_context_recovers(ctx, variant):
    c = configs.penning_1k(n=4096, seed=5).clouds[0]
    fp = configs.penning_field(quad=(0.5, configs.nu_c(132.905), 0.0, 0.0, 1.0), delta=1e3)
    ctx.set_coulomb_variant(variant)  # -1: automatic (plain shape here), 9: k-d ordered
    ctx.set_fused(False)              # the tiled kernels, whose copy ring is under test
    try:
        b = Batch(ctx, [len(c.mass)], [fp], [configs.ode(1e-9, 1e-15, 1e-9, 1e-6)],
                  SG_PREC_FP32C)
        b.upload(c.pos, c.vel, c.mass, c.charge)
        ref_info, st = b.step()
        assert st == abi.SG_OK
        ref_p, ref_v = b.download()

        b.upload(c.pos, c.vel, c.mass, c.charge)
        ctx.set_wait_test(0, 1000)       # every block gives up at its first tile after 1 ms
        info, st = b.step(raise_on_error=False)
        assert st == abi.SG_TIMEOUT
        assert info[0]["status"] == abi.SG_TIMEOUT and info[0]["steps"] == 0
        assert info[0]["t"] == 0.0       # nothing was committed
        p, v = b.download()
        assert np.array_equal(p, c.pos) and np.array_equal(v, c.vel)

        ctx.set_wait_test(-1)
        b.upload(c.pos, c.vel, c.mass, c.charge)
        info, st = b.step()
        assert st == abi.SG_OK and info[0]["status"] == abi.SG_OK
        assert info[0]["steps"] == ref_info[0]["steps"] == 1
        assert info[0]["t"] == ref_info[0]["t"]
        p, v = b.download()
        assert np.array_equal(p, ref_p) and np.array_equal(v, ref_v)
    finally:
        ctx.set_coulomb_variant(-1)
        ctx.set_fused(True)
