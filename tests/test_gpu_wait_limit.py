"""The bounded barrier waits of the mixed form's bulk-tensor stencil give up with an error status.

With a wait limit of zero attempts the stencil's barrier waits give up before looking: the CTAs
record the timeout, wait (with the default limit) for the copies they issued and return, and
the library reports MITHRA_ERR_STATE instead of hanging.  No GPU fault is involved: every copy
completes, only the wait that looked for it gave up early."""
import pytest

import mithra_gb300 as mg
from tests.conftest import job

pytestmark = pytest.mark.gpu


def test_stencil_wait_timeout_is_reported(gpu_available):
    s = mg.Setup.from_job(job("kat-small.job"))
    ctx = mg.Context.from_setup(s, mg.FP32)
    ctx.run(1)  # normal limit: fine
    ctx.set_wait_limit(0)
    with pytest.raises(mg.MithraError, match="wait timed out") as e:
        ctx.run(1)
    assert "status -4" in str(e.value)
    ctx.close()
    # another context on the same device is unaffected
    c2 = mg.Context.from_setup(s, mg.FP32)
    c2.run(2)
    c2.synchronize()
    c2.close()
