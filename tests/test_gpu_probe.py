"""The shared-memory atomic roof the bench reports the sieve stages'
rates against (gbc_smem_atomic_peak: conflict-free atomicAnd throughput)."""
import pytest

import gbc

pytestmark = pytest.mark.gpu


def test_smem_atomic_probe():
    per_s, per_clk = gbc.smem_atomic_peak()
    # at most one atomic per lane of each SM sub-partition per clock
    assert per_s > 1e11 and 1.0 < per_clk <= 128.0
