"""The library's per-cell constitutive algebra against the oracle, on the CPU.

``rheotool_gb300/csrc/constitutive_cell.cuh`` holds the FP64 theta source
(decomposeGradU plus the model source, constitutiveEq.C:323-358 and each
``*Log.C``) and tau of every log model as host-and-device functions: the
kernels inline them, and ``tests/host/model_cells.cu`` builds the same
source for the host.  This test compares that host build with the oracle's
restatement (``or_theta_source``, ``or_tau_cells``) on random cells: random
symmetric theta (eigenvalues of A = exp(theta) from e^-1.5 to e^1.5) and
random velocity gradients.  The GPU runs the same source, so a model that
passes here differs from the oracle on the device only through the
compiler's fused multiply-adds and the device math library.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import pyoracle
from rheotool_gb300 import abi
from rheotool_gb300.case import Model

HERE = os.path.dirname(os.path.abspath(__file__))
NVCC = next((c for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc"))
             if c and os.path.exists(c)), None)

MODELS = [
    ("Oldroyd-BLog", {}),
    ("GiesekusLog", {"alpha": 0.3}),
    ("PTTLog", {"epsilon": 0.25, "zeta": 0.1}),
    ("PTTLog", {"epsilon": 0.25, "destructionFunctionType": "exponential"}),
    ("PTTLog", {"epsilon": 0.25, "zeta": 0.1, "destructionFunctionType": "generalized", "alpha": 0.8, "beta": 1.2}),
    ("PTTLog", {"epsilon": 0.5, "destructionFunctionType": "generalized", "alpha": 1.5, "beta": 0.7,
                "maxIterMittagLeffler": 12}),
    ("FENE-PLog", {"L2": 100.0}),
    ("FENE-CRLog", {"L2": 20.0}),
    ("Rolie-PolyLog", {"lambdaR": 0.2, "beta": 0.5, "delta": -0.5}),
    ("Rolie-PolyLog", {"lambdaR": 0.3, "beta": 0.3, "delta": -0.5, "chiMax": 5.0}),
    ("XPomPomLog", {"lambdaS": 0.4, "q": 2.0, "alpha": 0.15, "n": 0.0}),
    ("XPomPomLog", {"lambdaS": 0.25, "q": 5.0, "alpha": 0.1, "n": 1.5}),
    ("WhiteMetznerCYLog", {"K": 0.5, "a": 2.0, "n": 0.6}),
    ("WhiteMetznerCYLog", {"K": 2.0, "a": 0.8, "n": 0.3}),
]


@pytest.fixture(scope="module")
def cells(tmp_path_factory):
    if NVCC is None:
        pytest.skip("nvcc not found")
    out = str(tmp_path_factory.mktemp("mc") / "libmodelcells.so")
    subprocess.check_call([NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O2",
                           "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-shared", "-o", out,
                           os.path.join(HERE, "host", "model_cells.cu")])
    lib = C.CDLL(out)
    dp = C.POINTER(C.c_double)
    lib.mc_theta_source.argtypes = [C.POINTER(abi.rt_model_params), C.c_int, dp, dp, dp, dp, dp, dp]
    lib.mc_tau.argtypes = [C.POINTER(abi.rt_model_params), C.c_int, dp, dp, dp, dp]
    return lib


def random_cells(n, seed):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.normal(size=(n, 3, 3)))
    mu = rng.uniform(-1.5, 1.5, size=(n, 3))
    th = np.einsum("nij,nj,nkj->nik", Q, mu, Q)
    theta = np.stack([th[:, 0, 0], th[:, 0, 1], th[:, 0, 2], th[:, 1, 1], th[:, 1, 2], th[:, 2, 2]], axis=1)
    eigVals, eigVecs = pyoracle.eig(theta)
    L = rng.normal(size=(n, 9))
    return L, eigVecs, eigVals, theta


def soa(a):
    return np.ascontiguousarray(a.T)


@pytest.mark.parametrize("model,kw", MODELS)
def test_cell_algebra_matches_oracle(cells, model, kw):
    mp = Model(model, rho=1.0, etaS=0.3, etaP=0.7, lambda_=0.8, **kw).to_c()
    n = 512
    L, eigVecs, eigVals, theta = random_cells(n, 20261204)
    rhs_o, fP_o = pyoracle.theta_source(mp, L, eigVecs, eigVals, theta)

    Ls, Rs, es, ts = (soa(a) for a in (L, eigVecs, eigVals, theta))
    rhs_s, fP_g = np.zeros((6, n)), np.zeros(n)
    cells.mc_theta_source(C.byref(mp), n, abi.dptr(Ls), abi.dptr(Rs), abi.dptr(es), abi.dptr(ts),
                          abi.dptr(rhs_s), abi.dptr(fP_g))
    rhs_g = rhs_s.T
    assert np.all(np.isfinite(rhs_o))
    assert np.max(np.abs(rhs_g - rhs_o)) <= 1e-13 * np.max(np.abs(rhs_o))
    if model in ("FENE-PLog", "FENE-CRLog", "WhiteMetznerCYLog"):
        assert np.max(np.abs(fP_g - fP_o)) <= 1e-14 * np.max(np.abs(fP_o))

    tau_o = pyoracle.tau_cells(mp, eigVecs, eigVals, fP_o)
    tau_s = np.zeros((6, n))
    cells.mc_tau(C.byref(mp), n, abi.dptr(Rs), abi.dptr(es), abi.dptr(fP_o), abi.dptr(tau_s))
    assert np.max(np.abs(tau_s.T - tau_o)) <= 1e-14 * np.max(np.abs(tau_o))


def test_generalized_ptt_with_unit_alpha_beta_is_the_exponential(cells):
    """Gamma(1) E_{1,1}(z) = exp(z): the generalized function with alpha =
    beta = 1 gives the exponential PTT source to the series tolerance."""
    L, eigVecs, eigVals, theta = random_cells(256, 11)
    kw = dict(rho=1.0, etaS=0.3, etaP=0.7, lambda_=0.8, epsilon=0.3)
    gen = Model("PTTLog", destructionFunctionType="generalized", alpha=1.0, beta=1.0, **kw).to_c()
    exp_ = Model("PTTLog", destructionFunctionType="exponential", **kw).to_c()
    rg, _ = pyoracle.theta_source(gen, L, eigVecs, eigVals, theta)
    re, _ = pyoracle.theta_source(exp_, L, eigVecs, eigVals, theta)
    assert np.max(np.abs(rg - re)) <= 1e-11 * np.max(np.abs(re))


def test_whitemetznercy_factor_is_the_carreau_yasuda_law(cells):
    """etaP(gd)/lambda(gd) kept for tau equals etaP/lambda: with m = n, K = L
    and a = b both carry the same factor (1 + (K gd)^a)^((n-1)/a)."""
    mp = Model("WhiteMetznerCYLog", etaP=0.7, lambda_=0.8, K=0.5, a=2.0, n=0.6).to_c()
    L, eigVecs, eigVals, theta = random_cells(64, 7)
    _, fP = pyoracle.theta_source(mp, L, eigVecs, eigVals, theta)
    assert np.allclose(fP, 0.7 / 0.8, rtol=1e-14)
