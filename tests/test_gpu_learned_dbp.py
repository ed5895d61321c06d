"""Learned DBP against plain many-step DBP on the precision-study link, and
what the correction CNN adds.

The 5-channel WDM link (32 GBaud 16QAM on a 50 GHz grid, 16 samples/symbol
of the total band, 20 x 80 km SSMF, ADAPTIVE 0.005 rad / 1 km, EDFA NF 5 dB
with ASE), centre channel at 2 samples/symbol, at -2, +2 and +4 dBm per
channel: training and test sets of 16 realizations x 2^15 symbols each,
generated by the GPU split step.

* The learned DBP at 4 steps per span (per-step FIR dispersion filters and
  nonlinear gains trained by the hand-written backward kernels, focss_ldbp_*)
  must score within 0.1 dB of plain 100-steps/span DBP (backward_propagation,
  src/tasks/systems.cpp:73-91) in at most a tenth of its GPU time, and above
  plain DBP at the same 4 steps per span.
* The correction CNN on the learned-DBP symbols and their perturbation
  triplets (focss_cnn_*, tensor-core kernels) must add more than 0.31 dB at
  +4 dBm/ch, where nonlinearity is strongest, and lose nothing (0.02 dB) at
  +2 dBm/ch and below; it is kept only if it lowers the error on held-out
  training realizations.
"""
import pytest

from focss_gb300 import links

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("power_dbm", [-2.0, 2.0, 4.0])
def test_learned_dbp_and_cnn_on_the_wdm_link(ctx, power_dbm):
    link = links.Link()
    r = links.learned_vs_plain(link, power_dbm, n_symbols=1 << 15, batch=16, seed=int(100 + 10 * power_dbm),
                               ctx=ctx, plain_steps=(4, 100))
    print("\nWDM centre channel %+.0f dBm/ch: %s" % (
        power_dbm, {k: (round(v["q_db"], 3), round(v["ms"], 2)) for k, v in r.items()}))
    l4, c4, p4, p100 = r["learned_4"], r["learned_4_cnn"], r["plain_4"], r["plain_100"]
    assert l4["q_db"] > p100["q_db"] - 0.1
    assert l4["ms"] < p100["ms"] / 10
    assert l4["q_db"] > p4["q_db"]
    if power_dbm >= 4.0:
        assert c4["q_db"] > l4["q_db"] + 0.31
    else:
        assert c4["q_db"] > l4["q_db"] - 0.02
