"""Edge cases of the device path against the oracle: a ragged mesh (10 x 13 transverse nodes,
rows padded to 16, centred off axis) in both forms, and a march with no particles at all."""
import numpy as np
import pytest

import mithra_gb300 as mg
from oracle import pyoracle as po
from tests.conftest import job, rel_l2

pytestmark = pytest.mark.gpu


def oracle_march(s, n):
    m = s.meta()
    anp1, an, anm1 = s.fields()
    o = po.OracleRun(m, an, anm1, anp1, s.particles(), solver=0, order=2)
    for _ in range(n):
        o.step()
    return o


@pytest.mark.parametrize("precision,rtol", [(mg.FP64, 1e-10), (mg.FP32, 2e-4)])
def test_ragged_mesh_march_matches_oracle(gpu_available, precision, rtol):
    s = mg.Setup.from_job(job("kat-small-ragged.job"))
    assert (int(s.meta()["N0"]), int(s.meta()["N1"])) == (10, 13)
    o = oracle_march(s, 12)
    ctx = mg.Context.from_setup(s, precision)
    ctx.run_prelude()
    ctx.run(12)
    _, an, anm1 = ctx.download_fields()
    assert rel_l2(an, o.an) <= rtol and rel_l2(anm1, o.anm1) <= rtol
    assert ctx.download_particles().shape == o.particles.shape
    rows = ctx.power_rows().reshape(12, -1)
    ref = np.array([np.ravel(np.column_stack([zl, pg.reshape(len(zl), -1)])) for zl, pg in o.power_rows])
    assert np.abs(rows - ref).max() <= max(rtol, 1e-9) * 10 * np.abs(ref).max()


@pytest.mark.parametrize("precision", [mg.FP64, mg.FP32])
def test_march_without_particles(gpu_available, precision):
    """No particles: the graph steps run, nothing is deposited, the fields stay zero and the
    power rows are zero (the reference's loop over an empty list)."""
    s = mg.Setup.from_job(job("kat-small.job"))
    ctx = mg.Context.from_setup(s, precision)
    ctx.upload_particles(np.zeros((0, 11)))
    ctx.run(5)
    anp1, an, anm1 = ctx.download_fields()
    assert not np.any(an) and not np.any(anm1)
    assert ctx.download_particles().shape == (0, 11)
    assert not np.any(ctx.power_rows().reshape(5, -1)[:, 1:])
