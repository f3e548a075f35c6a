"""The random-access probe (ltp_probe_random_access) that gives the batch
kernels their random-access roofline: it runs, rejects bad arguments, and
orders as the memory hierarchy says (an L2-sized array is faster to load
from at random than an HBM-sized one)."""
import pytest

import ltpmg_gb300 as G

pytestmark = pytest.mark.gpu


def test_probe_rates_and_arguments():
    small = G.lib.probe_random_access(0, 8 << 20, G.lib.PROBE_LOAD)
    big = G.lib.probe_random_access(0, 1 << 30, G.lib.PROBE_LOAD)
    atom = G.lib.probe_random_access(0, 8 << 20, G.lib.PROBE_ATOMIC)
    red = G.lib.probe_random_access(0, 8 << 20, G.lib.PROBE_REDUCE)
    assert small > big > 1e9 and atom > 1e9 and red > 1e9
    for bad in ((0, 100, G.lib.PROBE_LOAD), (0, 1 << 20, 7)):
        with pytest.raises(G.LtpError):
            G.lib.probe_random_access(*bad)
