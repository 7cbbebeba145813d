"""GPU parity at the benchmark's own configurations, through the C ABI, against the
oracle on the same seeded inputs:

* GYRE nn_GYRE=25 (752 x 502 x 31), the mixed form on its default kernels (the
  TMA-staged tracer kernels) -- the configuration the headline is measured on;
* the ensemble: 64 members of GYRE nn_GYRE=5 (152 x 102 x 31) in one context,
  member index outermost, one launch per kernel for all members; four members
  spread over the ensemble are checked against their own oracle;
* a 250 x 300 x 56 slice of the synthetic shelf (z*, partial steps, FCT 4/4,
  iso-neutral diffusion, flux-form momentum, atmospheric pressure), FP64 and mixed.

Tolerances are those of tests/test_gpu_parity.py (normwise relative error per
field: 1e-12 in FP64; TOL32_FIELD / TOL32_SPG in the mixed form). The pointwise
largest relative error, the largest distance in FP64 ulps and the fraction of
identical values of every field are recorded (tests/harness.py REPORT) and written
to $NEMO_PARITY_REPORT when that is set.
"""
import numpy as np
import pytest

from harness import ACC_2D, Pair

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32_FIELD = 5e-6
TOL32_SPG = 2e-3


def tol(prec, kind):
    if prec == "fp64":
        return TOL64
    return {"field": TOL32_FIELD, "spg": TOL32_SPG}[kind]


@pytest.fixture(autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _compare_step(p, prec):
    p.compare("TSA", p.s4, tol(prec, "field"))
    p.compare("AH_WSLP2", p.s3, tol(prec, "field"))
    for n in ("UA", "VA", "UN", "VN"):
        p.compare(n, p.s3, tol(prec, "spg"))
    for n in ACC_2D:
        p.compare(n, p.s2, tol(prec, "spg"))


def test_gyre25_one_step_mixed_tma():
    """One hot-path step of the benchmark workload in the mixed form, on the kernels
    the benchmark runs (TMA-staged iso-neutral fluxes and FCT stages)."""
    p = Pair(nn=25, prec="mixed", seed=14)
    p.bind_hotpath()
    p.ctx.set_timing(True)  # per-kernel launch counts: which kernels ran
    p.ora[0].stp_hotpath(5)
    p.ctx.stp_hotpath(5)
    p.ctx.synchronize()
    ran = p.ctx.get_kernel_timing()
    p.ctx.set_timing(False)
    assert "iso_flux_tma" in ran and ("fct_a_tma" in ran or "fct_fused" in ran), ran
    _compare_step(p, "mixed")


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_ensemble_64_members(prec):
    """64 members of GYRE nn_GYRE=5, each with its own seeded perturbation, two
    steps (the second a graph replay); members 0, 21, 42, 63 against their oracle."""
    p = Pair(nn=5, prec=prec, seed=13, nmem=64, sample=(0, 21, 42, 63))
    p.bind_hotpath()
    for kt in (5, 6):
        for o in p.ora:
            o.stp_hotpath(kt)
        p.ctx.stp_hotpath(kt)
        p.ctx.synchronize()
    _compare_step(p, prec)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_shelf_slice(prec):
    """A 250 x 300 x 56 slice of the synthetic shelf, two steps from an Euler start:
    z* variable volume, partial bottom cells, FCT 4/4, iso-neutral diffusion, EEN
    vorticity, flux-form momentum, atmospheric pressure, nn_baro = 30."""
    from nemo_gpu import shelf
    dom = shelf.domain(250, 300, 56, seed=3)
    nam = shelf.namelist(neuler=0)
    st = shelf.state(dom, nam, seed=4)
    p = Pair(prec=prec, dom=dom, nam=nam, states=[st])
    p.bind_hotpath()
    for n in ("GTSU", "GTSV", "SSH_IB"):
        p.bind(n)
    for kt in (1, 2):
        p.ora[0].stp_hotpath(kt)
        p.ctx.stp_hotpath(kt)
        p.ctx.synchronize()
    _compare_step(p, prec)
    assert np.abs(p.host[0]["TSA"]).max() > 0
