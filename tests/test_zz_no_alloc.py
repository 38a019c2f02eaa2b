"""The entry point that allocates no device memory (gf_nll_exp_noalloc).

It serves callers that cannot allocate device memory while they evaluate the
likelihood.  Checked here through the C ABI against the engine's regular
gf_nll_grad on the same ExpPdf data, with the tolerances of the other parity
tests (NLL 1e-6 relative; gradient within 1e-3 sqrt(n)), on two calls in a
row.  The device buffers of the test itself come from torch; the entry point
under test allocates nothing.  This file is collected last on purpose.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_matches_engine_on_two_calls():
    torch = pytest.importorskip("torch")
    import goofit_gb300 as gf
    from goofit_gb300 import _abi as A
    from goofit_gb300 import workloads as W

    n = 100_000
    wl = W.make_c1(n, seed=21)
    nodes, params, obs = wl.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    eng = gf.Engine("mixed")
    eng.set_tree(nodes, olist, len(params), [1])
    eng.upload(wl.data.to_numpy())

    x = torch.tensor(wl.data.to_numpy()[0], dtype=torch.float32, device="cuda:0")
    out = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    L = A.lib()
    for alpha in (-0.7, -0.45):
        rc = L.gf_nll_exp_noalloc(C.c_void_p(x.data_ptr()), n, alpha, 0.0, 10.0, C.c_void_p(out.data_ptr()), None)
        assert rc == 0, L.gf_noalloc_last_error()
        torch.cuda.synchronize()
        got_nll, got_g = out.cpu().tolist()
        ref_nll, ref_g = eng.nll_grad([alpha])
        assert got_nll == pytest.approx(ref_nll, rel=1e-6)
        assert got_g == pytest.approx(ref_g[0], rel=1e-5, abs=1e-3 * math.sqrt(n))


def test_noalloc_rejects_sizes_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    from goofit_gb300 import _abi as A
    L = A.lib()
    out = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    x = torch.zeros(16, dtype=torch.float32, device="cuda:0")
    # the pointer is never read: the size check fails first
    rc = L.gf_nll_exp_noalloc(C.c_void_p(x.data_ptr()), 8_388_609, -0.5, 0.0, 10.0, C.c_void_p(out.data_ptr()), None)
    assert rc == A.GF_ERR_INVALID
    assert b"8388608" in L.gf_noalloc_last_error()
