"""The allocation-free global sum (nemo_gpu_glob_sum_noalloc) against the context
entry point nemo_gpu_glob_sum, through the C ABI.

nemo_gpu_glob_sum_noalloc exists for callers that cannot allocate device memory
when they need a conservation sum (inside an open CUDA stream capture, under a
host runtime that owns all device memory, or with a device footprint fixed at
start-up); it keeps its partial sums in a static device array instead. This file
is collected last so that a run stopping at the first failure has already run
every other test; it also passes on its own in a fresh process.
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
    tmask_i = ora.Oracle(dom, nam).array("tmask_i")
    mask = torch.from_numpy(np.ascontiguousarray(tmask_i.ravel(order="F"))).to("cuda")
    return dom, ctx, mask


def _noalloc(lib, t, mask, dom, nk, nmem, is64, out):
    return lib.nemo_gpu_glob_sum_noalloc(C.c_void_p(t.data_ptr()), C.c_void_p(mask.data_ptr()), dom["jpi"],
                                         dom["jpj"], nk, nmem, is64, None, C.c_void_p(out.data_ptr()))


@pytest.mark.parametrize("is64", [1, 0])
def test_noalloc_glob_sum_matches_context_glob_sum(is64):
    dom, ctx, mask = _setup(nmem=3)
    jpi, jpj, jpk = dom["jpi"], dom["jpj"], dom["jpk"]
    rng = np.random.default_rng(7)
    dtype = torch.float64 if is64 else torch.float32
    out = torch.empty(3, dtype=torch.float64, device="cuda")
    for call in range(2):                       # two calls in a row, different data
        x = rng.standard_normal(3 * jpi * jpj * jpk) * 10.0 ** rng.integers(-6, 7, 3 * jpi * jpj * jpk)
        t = torch.from_numpy(x).to("cuda", dtype)
        ref = ctx.glob_sum(t, jpk)
        out.fill_(float("nan"))
        st = _noalloc(ctx.lib, t, mask, dom, jpk, 3, is64, out)
        assert st == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        for m in range(3):
            assert abs(got[m] - ref[m]) <= 4 * np.spacing(abs(ref[m])), (call, m, got[m], ref[m])


def test_noalloc_glob_sum_rejects_too_many_members():
    dom, ctx, mask = _setup(nmem=1)
    t = torch.zeros(dom["jpi"] * dom["jpj"], dtype=torch.float64, device="cuda")
    out = torch.zeros(65, dtype=torch.float64, device="cuda")
    assert _noalloc(ctx.lib, t, mask, dom, 1, 65, 1, out) == NEMO_ERR_ARG
