"""Host copies through the C ABI (nemo_gpu_field_upload / nemo_gpu_field_download)
overlapped on the context's copy streams give the same results as fully serialised
copies: each step uploads new inputs, runs the hot path and downloads its outputs,
once with no synchronisation until the end and once synchronising after every call.
"""
import pytest

from harness import Pair

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

INS = ("TSB", "TSN", "UN", "VN", "UA", "VA")
OUTS = ("TSA", "UA", "VA", "UN", "VN")


@pytest.fixture(autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _run(prec, serialise, nsteps=3):
    p = Pair(nn=2, prec=prec, seed=21, neuler=0)
    p.bind_hotpath()
    gen = torch.Generator().manual_seed(5)
    ins = {}
    for n in INS:
        base = p.dev[n].detach().cpu()
        ins[n] = []
        for s in range(nsteps):  # a different input every step
            h = torch.empty(base.numel(), dtype=base.dtype, pin_memory=True)
            h.copy_(base.reshape(-1) * (1.0 + 0.01 * s) + 1e-3 * torch.randn(base.numel(), generator=gen).to(base.dtype))
            ins[n].append(h)
    outs = {n: [torch.empty(p.dev[n].numel(), dtype=p.dev[n].dtype, pin_memory=True) for _ in range(nsteps)]
            for n in OUTS}
    for s in range(nsteps):
        for n in INS:
            p.ctx.upload(n, ins[n][s])
            if serialise:
                p.ctx.synchronize()
        p.ctx.stp_hotpath(3 + s)
        if serialise:
            p.ctx.synchronize()
        for n in OUTS:
            p.ctx.download(n, outs[n][s])
            if serialise:
                p.ctx.synchronize()
    p.ctx.synchronize()
    return outs


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_overlapped_copies_match_serialised(prec):
    a = _run(prec, serialise=False)
    b = _run(prec, serialise=True)
    for n in OUTS:
        for s, (x, y) in enumerate(zip(a[n], b[n])):
            assert torch.equal(x, y), f"{n} step {s}: overlapped copies differ from serialised ones"


@pytest.mark.parametrize("nn", [1, 3])
def test_upload_then_download_without_a_step(nn):
    """A field of 1 MB or more (tsb at nn_GYRE=3) is staged on the device and copied
    into the field by the next work that reads it, a smaller one (nn_GYRE=1) goes
    straight into place; either way a download before any such work returns the
    uploaded values, and of two uploads of a field without work between them the
    later one wins."""
    p = Pair(nn=nn, prec="mixed", seed=3)
    p.bind_hotpath()
    n = p.dev["TSB"].numel()
    first = torch.arange(n, dtype=torch.float32).pin_memory()
    second = (torch.arange(n, dtype=torch.float32) * 0.5 + 1.0).pin_memory()
    got = torch.empty(n, dtype=torch.float32).pin_memory()
    p.ctx.upload("TSB", first)
    p.ctx.download("TSB", got)
    p.ctx.synchronize()
    assert torch.equal(got, first)
    p.ctx.upload("TSB", first)
    p.ctx.upload("TSB", second)
    p.ctx.download("TSB", got)
    p.ctx.synchronize()
    assert torch.equal(got, second)
    # and the field itself (read through torch after a synchronize) holds it too
    assert torch.equal(p.dev["TSB"].detach().reshape(-1).cpu(), second)
