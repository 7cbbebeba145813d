"""The allocation-free global sum (nemo_gpu_glob_sum_noalloc) against the context
entry point nemo_gpu_glob_sum and the oracle's glob_sum, through the C ABI.

nemo_gpu_glob_sum_noalloc exists for callers that cannot allocate device memory
when they need a conservation sum: a host model whose device memory is owned by
another runtime (an OpenACC or CUDA Fortran data region, a coupler's allocator)
that must not see allocations behind its back, or a set-up whose device footprint
is fixed at start-up. It keeps its partial sums in a static device array instead,
so it serves at most 64 members per call. This file is collected last so that a
run stopping at the first failure has already run every other test; it also
passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

NEMO_ERR_ARG = 1


@pytest.fixture(autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _setup(nmem=3):
    from nemo_gpu import api, gyre
    from oracle import ora
    dom = gyre.domain(2)
    nam = gyre.namelist()
    ctx = api.Context(dom, nam, nmembers=nmem, prec="fp64")
    o = ora.Oracle(dom, nam)
    tmask_i = o.array("tmask_i")
    mask = torch.from_numpy(np.ascontiguousarray(tmask_i.ravel(order="F"))).to("cuda")
    return dom, ctx, mask, o


def _noalloc(lib, t, mask, dom, nk, nmem, is64, out):
    return lib.nemo_gpu_glob_sum_noalloc(C.c_void_p(t.data_ptr()), C.c_void_p(mask.data_ptr()), dom["jpi"],
                                         dom["jpj"], nk, nmem, is64, None, C.c_void_p(out.data_ptr()))


def _fields(rng, nmem, n, is64):
    """nmem fields of n values spanning 13 decades (exponents -6..6), rounded to the
    element type so the oracle sums exactly the values the GPU reads"""
    x = rng.standard_normal(nmem * n) * 10.0 ** rng.integers(-6, 7, nmem * n)
    if not is64:
        x = x.astype(np.float32).astype(np.float64)
    return x


@pytest.mark.parametrize("nmem", [3, 64])
@pytest.mark.parametrize("is64", [1, 0])
def test_noalloc_glob_sum_matches_context_glob_sum(is64, nmem):
    dom, ctx, mask, o = _setup(nmem=nmem)
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    n3 = jpi * jpj * jpk
    rng = np.random.default_rng(7 + nmem)
    dtype = torch.float64 if is64 else torch.float32
    out = torch.empty(nmem, dtype=torch.float64, device="cuda")
    for call in range(2):                       # two calls in a row, different data
        x = _fields(rng, nmem, n3, is64)
        t = torch.from_numpy(x).to("cuda", dtype)
        ref = ctx.glob_sum(t, jpk)
        out.fill_(float("nan"))
        st = _noalloc(ctx.lib, t, mask, dom, jpk, nmem, is64, out)
        assert st == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        for m in range(nmem):
            assert abs(got[m] - ref[m]) <= 4 * np.spacing(abs(ref[m])), (call, m, got[m], ref[m])
        # against the oracle's DDPDD sum (lib_fortran.F90:300-332) of the same member
        for m in (0, nmem // 2, nmem - 1):
            fm = np.asfortranarray(x[m * n3:(m + 1) * n3].reshape((jpi, jpj, jpk), order="F"))
            r = o.glob_sum(fm)
            assert abs(got[m] - r) <= 4 * np.spacing(abs(r)), (call, m, got[m], r)


def test_noalloc_glob_sum_rejects_too_many_members():
    dom, ctx, mask, _ = _setup(nmem=1)
    t = torch.zeros(dom["jpi"] * dom["jpj"], dtype=torch.float64, device="cuda")
    out = torch.zeros(65, dtype=torch.float64, device="cuda")
    assert _noalloc(ctx.lib, t, mask, dom, 1, 65, 1, out) == NEMO_ERR_ARG
