"""The entry point that allocates no device memory (gf_nll_exp_noalloc).

It serves callers that cannot allocate device memory while they evaluate the
likelihood: a host whose device memory is owned by another allocator or by a
fixed budget, and latency-critical code in which cudaMalloc / cudaFree may
synchronise the device.  Checked here through the C ABI against the engine's
regular gf_nll_grad and against the FP64 oracle on the same ExpPdf data, with
the tolerances of the other parity tests (NLL 1e-6 relative; gradient within
1e-3 sqrt(n)), on two calls in a row, at a small size and at the largest size
its fixed scratch array allows; a fine scan of alpha checks that the NLL moves
smoothly (no steps from an FP32 normalisation factor).  The device buffers of
the test itself come from torch; the entry point under test allocates nothing.
This file is collected last on purpose.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_EVENTS = 8_388_608


def _call(L, x, n, alpha, out):
    rc = L.gf_nll_exp_noalloc(C.c_void_p(x.data_ptr()), n, alpha, 0.0, 10.0, C.c_void_p(out.data_ptr()), None)
    assert rc == 0, L.gf_noalloc_last_error()


@pytest.mark.parametrize("n", [100_000, MAX_EVENTS])
def test_noalloc_matches_engine_and_oracle_on_two_calls(n):
    torch = pytest.importorskip("torch")
    import goofit_gb300 as gf
    from goofit_gb300 import _abi as A
    from goofit_gb300 import workloads as W
    from oracle import oracle as O

    wl = W.make_c1(n, seed=21)
    soa = wl.data.to_numpy()
    nodes, params, obs = wl.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    eng = gf.Engine("mixed")
    eng.set_tree(nodes, olist, len(params), [1])
    eng.upload(soa)

    x = torch.tensor(soa[0], dtype=torch.float32, device="cuda:0")
    out = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    L = A.lib()
    for alpha in (-0.7, -0.45):
        _call(L, x, n, alpha, out)
        torch.cuda.synchronize()
        got_nll, got_g = out.cpu().tolist()
        ref_nll, ref_g = eng.nll_grad([alpha])
        assert got_nll == pytest.approx(ref_nll, rel=1e-6)
        assert got_g == pytest.approx(ref_g[0], rel=1e-5, abs=1e-3 * math.sqrt(n))
        # the oracle sees the FP32 events the kernel reads and alpha rounded to FP32, as the kernel does
        a32 = float(np.float32(alpha))
        xs = soa[0].astype(np.float32).astype(np.float64)[None, :]
        o_nll = O.nll(nodes, olist, [a32], xs)
        assert got_nll == pytest.approx(o_nll, rel=1e-6)
        o_g = O.fd_grad(nodes, olist, [a32], xs, [0], h=1e-5)[0]
        assert got_g == pytest.approx(o_g, rel=1e-5, abs=1e-3 * math.sqrt(n))
    eng.close()


def test_noalloc_nll_is_smooth_in_alpha():
    """Steps of a few FP32 ulps in alpha at the largest size: the difference to the FP64 oracle must stay
    constant to well below MIGRAD's up = 0.5 (a normalisation factor rounded to FP32 per event moved the
    NLL by up to n 2^-24 = 0.5 in steps)."""
    torch = pytest.importorskip("torch")
    from goofit_gb300 import _abi as A
    from goofit_gb300 import workloads as W
    from oracle import oracle as O

    n = MAX_EVENTS
    wl = W.make_c1(n, seed=22)
    soa = wl.data.to_numpy()
    nodes, params, obs = wl.pdf._flatten()
    olist = [(o.lowerlimit, o.upperlimit, o.numbins, int(o.is_event_number)) for o in obs]
    xs = soa[0].astype(np.float32).astype(np.float64)[None, :]
    x = torch.tensor(soa[0], dtype=torch.float32, device="cuda:0")
    out = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    L = A.lib()
    a = np.float32(-0.6)
    diffs, incs, grads = [], [], []
    prev = None
    for _ in range(12):
        _call(L, x, n, float(a), out)
        torch.cuda.synchronize()
        got, g = out.cpu().tolist()
        ref = O.nll(nodes, olist, [float(a)], xs)
        diffs.append(got - ref)
        grads.append(g)
        if prev is not None:
            incs.append((got - prev[0], ref - prev[1]))
        prev = (got, ref)
        for _ in range(3):
            a = np.nextafter(a, np.float32(0.0))
    diffs = np.array(diffs)
    assert np.ptp(diffs) < 0.05, diffs
    for got_inc, ref_inc in incs:
        assert got_inc == pytest.approx(ref_inc, abs=0.05)
    assert all(gv > 0 for gv in grads) or all(gv < 0 for gv in grads)


def test_noalloc_rejects_sizes_and_alphas_it_cannot_serve():
    torch = pytest.importorskip("torch")
    from goofit_gb300 import _abi as A
    L = A.lib()
    out = torch.zeros(2, dtype=torch.float64, device="cuda:0")
    x = torch.zeros(16, dtype=torch.float32, device="cuda:0")
    # the pointer is never read: the size check fails first
    rc = L.gf_nll_exp_noalloc(C.c_void_p(x.data_ptr()), MAX_EVENTS + 1, -0.5, 0.0, 10.0,
                              C.c_void_p(out.data_ptr()), None)
    assert rc == A.GF_ERR_INVALID
    assert b"8388608" in L.gf_noalloc_last_error()
    # no finite, positive normalisation integral: rejected on the host before any launch
    for alpha in (float("nan"), float("inf"), 1e6):
        rc = L.gf_nll_exp_noalloc(C.c_void_p(x.data_ptr()), 16, alpha, 0.0, 10.0, C.c_void_p(out.data_ptr()), None)
        assert rc == A.GF_ERR_INVALID, alpha
        assert b"normalisation" in L.gf_noalloc_last_error()
