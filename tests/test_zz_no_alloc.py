"""drmlt_compute_gaussian_noalloc: the FP64 H2MC Gaussian for callers that cannot
allocate device memory (they own every device buffer, e.g. carved from their own
pool, and the library must not call cudaMalloc behind their back).

The test owns the device buffers (torch tensors), calls the entry point twice in
a row through the C ABI -- the second call reuses the library's fixed scratch
array left over from the first -- and checks each result against
drmlt_compute_gaussian (which allocates its own temporaries) within the
Gaussian tolerance of the parity tests (1e-3 relative). It also checks that a
batch larger than the fixed scratch is rejected with DRMLT_E_ARG.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import golden

pytestmark = pytest.mark.gpu

MAX = 24
TOL = 1e-3  # Gaussian tolerance used by test_gpu_parity


def _inputs(recs):
    n = len(recs)
    dims = np.array([r["dim"] for r in recs], np.int32)
    ss = np.array([r["contrib"][0]["ss"] for r in recs], np.float32)
    grad = np.zeros((n, MAX), np.float32)
    hess = np.zeros((n, MAX * MAX), np.float32)
    for i, r in enumerate(recs):
        d = r["dim"]
        grad[i, :d] = r["grad"]
        hess[i, :d * d] = r["hess"]
    return dims, ss, grad, hess


def _noalloc(capi, torch, dims, ss, grad, hess, sigma, stream=None):
    dev = torch.device("cuda:0")
    n = len(dims)
    t_dims = torch.from_numpy(dims).to(dev)
    t_ss = torch.from_numpy(ss).to(dev)
    t_grad = torch.from_numpy(grad).to(dev)
    t_hess = torch.from_numpy(hess).to(dev)
    # poison the outputs: the entry point must overwrite every entry
    t_mean = torch.full((n, MAX), 7.0, dtype=torch.float64, device=dev)
    t_ic = torch.full((n, MAX * MAX), 7.0, dtype=torch.float64, device=dev)
    t_cv = torch.full((n, MAX * MAX), 7.0, dtype=torch.float64, device=dev)
    t_ld = torch.full((n,), 7.0, dtype=torch.float64, device=dev)
    if stream is None:
        stream = torch.cuda.current_stream(dev)
    torch.cuda.current_stream(dev).synchronize()  # inputs written before the side stream reads them
    rc = capi.lib().drmlt_compute_gaussian_noalloc(
        n, C.c_void_p(t_dims.data_ptr()), C.c_void_p(t_ss.data_ptr()), C.c_void_p(t_grad.data_ptr()),
        C.c_void_p(t_hess.data_ptr()), C.c_float(sigma), C.c_void_p(t_mean.data_ptr()),
        C.c_void_p(t_ic.data_ptr()), C.c_void_p(t_cv.data_ptr()), C.c_void_p(t_ld.data_ptr()),
        C.c_void_p(stream.cuda_stream))
    capi.check(rc)
    torch.cuda.synchronize(dev)
    return t_mean.cpu().numpy(), t_ic.cpu().numpy(), t_cv.cpu().numpy(), t_ld.cpu().numpy()


def _close(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.max(np.abs(b)), 1e-12)
    return np.max(np.abs(a - b)) / scale <= TOL


def test_noalloc_gaussian_matches_allocating_entry(renderers):
    torch = pytest.importorskip("torch")
    from drmlt import capi
    recs = golden("cfg1", "tech")
    assert recs, "golden fixture cfg1_tech missing"
    r = renderers("cfg1")
    sigma = r.options.perturb_stddev
    batches = [recs[:100], recs[100:][::-1]]  # two calls in a row, different contents
    side = torch.cuda.Stream()  # the second call runs on a stream other than torch's current one
    for batch, stream in zip(batches, (None, side)):
        dims, ss, grad, hess = _inputs(batch)
        mean, ic, cv, ld = _noalloc(capi, torch, dims, ss, grad, hess, sigma, stream)
        rm, ric, rcv, rld = r.compute_gaussian(dims, ss, grad, hess)
        for i in range(len(batch)):
            assert _close(mean[i], rm[i]) and _close(ic[i], ric[i]) and _close(cv[i], rcv[i]), i
            assert abs(ld[i] - rld[i]) <= TOL * max(1.0, abs(rld[i])), i


def test_noalloc_rejects_oversized_batch(built_lib):
    from drmlt import capi
    null = C.c_void_p(0)
    rc = capi.lib().drmlt_compute_gaussian_noalloc(257, null, null, null, null, C.c_float(0.01), null, null, null,
                                                   null, null)
    assert rc == -1
    assert b"exceeds" in capi.lib().drmlt_last_error()


def test_noalloc_allocates_nothing_and_flags_bad_dims(renderers):
    """After a first call (the per-device set-up), further calls leave the
    device's free memory unchanged; a record with an odd dimension gets zero
    outputs and a NaN log-determinant while its neighbours are computed."""
    torch = pytest.importorskip("torch")
    from drmlt import capi
    recs = golden("cfg1", "tech")[:8]
    r = renderers("cfg1")
    sigma = r.options.perturb_stddev
    dims, ss, grad, hess = _inputs(recs)
    dims[3] = 7  # odd: not a path dimension 2L
    dev = torch.device("cuda:0")
    ins = [torch.from_numpy(a).to(dev) for a in (dims, ss, grad, hess)]
    n = len(dims)
    outs = [torch.full((n, MAX), 7.0, dtype=torch.float64, device=dev),
            torch.full((n, MAX * MAX), 7.0, dtype=torch.float64, device=dev),
            torch.full((n, MAX * MAX), 7.0, dtype=torch.float64, device=dev),
            torch.full((n,), 7.0, dtype=torch.float64, device=dev)]
    ptrs = [C.c_void_p(t.data_ptr()) for t in ins[:4]]
    optrs = [C.c_void_p(t.data_ptr()) for t in outs]
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

    def call():
        capi.check(capi.lib().drmlt_compute_gaussian_noalloc(n, *ptrs, C.c_float(sigma), *optrs, stream))
        torch.cuda.synchronize(dev)

    call()
    free0, _ = torch.cuda.mem_get_info(dev)
    for _ in range(3):
        call()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0, (free0, free1)
    mean, ic, cv, ld = (t.cpu().numpy() for t in outs)
    assert np.isnan(ld[3])
    assert not mean[3].any() and not ic[3].any() and not cv[3].any()
    ok = [i for i in range(n) if i != 3]
    assert np.isfinite(ld[ok]).all()
    rm, _, _, rld = r.compute_gaussian(dims[ok], ss[ok], grad[ok], hess[ok])
    for j, i in enumerate(ok):
        assert _close(mean[i], rm[j]), i
        assert abs(ld[i] - rld[j]) <= TOL * max(1.0, abs(rld[j])), i
