"""mithra_gpu_power_sample_noalloc against mithra_gpu_power_sample, through the C ABI.

The no-allocation variant runs the same sample and reduction kernels with the per-block partial
sums in a fixed per-device array instead of the context's buffer, so on the same fields it must
log the same power rows.  The file is named to be collected last; it also passes alone."""
import numpy as np
import pytest

import mithra_gb300 as mg
from tests._golden import TAGS, load
from tests.conftest import job

pytestmark = pytest.mark.gpu

ROWS_RTOL = 1e-12   # same kernels and summation order: equal up to rounding of the row copy
STATIC_PARTIAL_MAX = 1 << 17


def primed_context(tag="kat-small-fd"):
    f = load(tag, "field")
    ctx = mg.Context.from_setup(mg.Setup.from_job(job(TAGS[tag][0])))
    ctx.upload_fields(f["anp1"], f["an"], f["anm1"])
    ctx.field_evaluate()
    return ctx


def test_noalloc_rows_equal_two_calls_in_a_row(gpu_available):
    ref, var = primed_context(), primed_context()
    for _ in range(2):
        ref.power_sample()
        var.power_sample_noalloc()
        ref.advance_time()
        var.advance_time()
    a, b = ref.power_rows(), var.power_rows()
    assert a.shape == b.shape and a.size > 0
    assert np.abs(a).max() > 0
    err = np.abs(a - b).max() / np.abs(a).max()
    assert err <= ROWS_RTOL, "power rows differ: %.3e relative to max |row|" % err


def test_noalloc_refuses_outputs_beyond_the_fixed_array(gpu_available):
    ctx = primed_context()
    nl, nf = 64, 4
    n_planes = STATIC_PARTIAL_MAX // nl + 1   # one block per plane on this grid
    rng = np.random.default_rng(7)
    ctx.set_power([dict(N=n_planes, Nl=nl, Nf=nf, pc=1.0, z=np.full(n_planes, -1e9),
                        tw_re=rng.standard_normal(nl * nf), tw_im=rng.standard_normal(nl * nf))])
    with pytest.raises(mg.MithraError, match="fixed array holds 131072"):
        ctx.power_sample_noalloc()


def test_noalloc_refuses_when_the_row_log_is_full(gpu_available):
    ctx = primed_context()
    with pytest.raises(mg.MithraError, match="row log full"):
        for _ in range(100000):
            ctx.power_sample_noalloc()
    rows = ctx.power_rows()
    assert rows.size > 0
    ctx.power_sample_noalloc()   # room again after the drain
