"""What the trained closure gains over the same LES without it (GPU).

The 512^3 forced DNS is deterministic for a given seed, so the test regenerates
the trajectory the committed network (spectraldns_gb300/data/closure_64.npz)
was trained on, box-filters it (ratio 8) every 10 steps, and runs the 64^3 LES
with and without the closure from snapshot 150 (held out: training used
snapshots 0-149) to snapshot 169.  Spectrum error = max over 1 <= k <= 20 of
the relative shell-spectrum error against the filtered DNS.  Bars: the closure
keeps the time-averaged spectrum within 5% and at most half the error without
it, and does better on the snapshot-mean error as well.
"""
import os

import pytest

pytestmark = pytest.mark.gpu

MODEL = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "spectraldns_gb300", "data",
                     "closure_64.npz")


def test_closure_beats_no_closure(built_lib):
    from spectraldns_gb300 import les as L
    data = L.harvest(512, 8, steps=1700, every=10, log=None)
    net, nm, scale = L.load_model(MODEL, (64, 64, 64))
    with_net = L.run_les(data, net, nm, 150, 170, 64, scale=scale)
    without = L.run_les(data, None, nm, 150, 170, 64)
    assert with_net["finite"] and without["finite"]
    e1, e0 = with_net["max_err_k<=20_time_avg_spectrum"], without["max_err_k<=20_time_avg_spectrum"]
    assert e1 < 0.05, e1
    assert e1 < 0.5 * e0, (e1, e0)
    assert with_net["max_err_k<=20_mean"] < without["max_err_k<=20_mean"]
