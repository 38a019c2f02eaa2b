"""The event-chunking autotuner: after the first evaluation the engine reports the chunk size it chose (a
multiple of 256 events); with GF_AUTOTUNE=0 it keeps the occupancy-derived size; either way the NLL and
gradient agree with the oracle (mixed tolerance 1e-6 relative)."""
import numpy as np
import pytest

import goofit_gb300 as gf
from goofit_gb300 import workloads as W
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _engine(wl):
    nodes, params, obs = wl.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    mask = [0 if v.fixed else 1 for v in params]
    eng = gf.Engine("mixed")
    eng.set_tree(nodes, olist, len(params), mask)
    eng.upload(wl.data.to_numpy())
    return eng, nodes, olist, np.array([v.value for v in params])


@pytest.mark.parametrize("tune", ["1", "0"])
def test_autotuned_chunking_keeps_the_nll(tune, monkeypatch):
    monkeypatch.setenv("GF_AUTOTUNE", tune)
    wl = W.make_c2(300_000, seed=12)
    eng, nodes, olist, pv = _engine(wl)
    assert eng.event_chunk() == 0          # no layout before the first evaluation
    v, g = eng.nll_grad(pv)
    chunk = eng.event_chunk()
    assert chunk >= 256 and chunk % 256 == 0
    ref = O.nll(nodes, olist, pv, wl.data.to_numpy())
    assert v == pytest.approx(ref, rel=1e-6)
    # a second engine on the same tree and size reuses the choice
    eng2, *_ = _engine(wl)
    eng2.nll_grad(pv)
    assert eng2.event_chunk() == chunk
