"""Temperature-dependent parameters (rheoTool's thermoFunctions), on the CPU.

The oracle's shift factors are checked against the published formulas
(thermoFunctions/<type>/<type>.C, multiply()).  Its temperature-dependent
correct() is checked against the isothermal correct() where the answer is
known exactly:
- Constant functions are the isothermal case.
- A uniform temperature is the isothermal case with the relaxation times
  and etaP multiplied by the factors.
- A temperature field that shifts etaP alone leaves theta alone and scales
  each cell's tau by its own factor.
"""
import copy

import numpy as np
import pytest

from rheotool_gb300.case import ThermoFunction, cavity_case

FUNCTIONS = [
    ThermoFunction("Constant"),
    ThermoFunction("Arrhenius", alpha=4000.0, T0=300.0),
    ThermoFunction("ArrheniusModified", alpha=0.02, T0=300.0),
    ThermoFunction("WLF", c1=8.86, c2=101.6, T0=300.0),
    ThermoFunction("VFT", A=500.0, B=-1.0, T0=150.0),
]

MODELS = [("Oldroyd-BLog", {}), ("GiesekusLog", {"alpha": 0.1}), ("PTTLog", {"epsilon": 0.25}),
          ("FENE-PLog", {"L2": 100.0}), ("FENE-CRLog", {"L2": 20.0}),
          ("Rolie-PolyLog", {"lambdaR": 0.2, "chiMax": 5.0}),
          ("XPomPomLog", {"lambdaS": 0.2, "q": 2.0, "alpha": 0.15}),
          ("WhiteMetznerCYLog", {"K": 1.0, "a": 2.0})]


def rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def model_cavity(model, kw, n=10):
    kw = dict(kw)
    late = {k: kw.pop(k) for k in ("beta", "n") if k in kw}
    case = cavity_case(n, model=model, Wi=0.8, dt=5e-3, **kw)
    for k, v in late.items():
        setattr(case.model, k, v)
    return case


def developed(case, steps=3):
    from oracle.pyoracle import Oracle
    o = Oracle(case)
    o.step(steps)
    return o.f.copy()


@pytest.mark.parametrize("fn", FUNCTIONS, ids=lambda f: f.type)
def test_oracle_thermo_factors_are_the_published_formulas(fn):
    import ctypes as C
    from oracle import pyoracle
    T = np.linspace(280.0, 420.0, 57)
    c = fn.to_c()
    got = np.array([pyoracle.lib().or_thermo_factor(C.byref(c), float(t)) for t in T])
    assert np.allclose(got, fn.factor(T), rtol=1e-14, atol=0.0)
    if fn.type in ("Arrhenius", "ArrheniusModified", "WLF"):
        # every shift is 1 at its reference temperature
        assert pyoracle.lib().or_thermo_factor(C.byref(c), fn.T0) == 1.0


def test_thermo_factor_values():
    """A few values worked by hand: Arrhenius alpha 4000 K from 300 K to
    400 K is exp(4000 (1/400 - 1/300)) = exp(-10/3); WLF with the universal
    constants 10 K above T0 is 10^(-88.6 / 111.6)."""
    assert np.isclose(FUNCTIONS[1].factor(400.0), np.exp(-10.0 / 3.0), rtol=1e-15)
    assert np.isclose(FUNCTIONS[3].factor(310.0), 10.0 ** (-88.6 / 111.6), rtol=1e-15)
    assert np.isclose(FUNCTIONS[2].factor(250.0), np.exp(1.0), rtol=1e-15)
    assert np.isclose(FUNCTIONS[4].factor(400.0), 10.0 ** (-1.0 + 2.0), rtol=1e-15)


def test_unknown_thermo_type_is_refused():
    with pytest.raises(ValueError):
        ThermoFunction("Eyring").to_c()


@pytest.mark.parametrize("model,kw", MODELS)
def test_oracle_constant_functions_are_the_isothermal_correct(model, kw):
    from oracle.pyoracle import Oracle
    case = model_cavity(model, kw)
    f0 = developed(case)
    a = Oracle(case, f0.copy())
    a.constitutive_correct()
    b = Oracle(case, f0.copy())
    b.constitutive_correct(T=np.full(case.mesh.nCells, 350.0))
    for name in ("theta", "tau", "eigVals", "eigVecs", "taub"):
        assert np.array_equal(getattr(a.f, name), getattr(b.f, name)), name


@pytest.mark.parametrize("model,kw", MODELS)
def test_oracle_uniform_temperature_scales_the_parameters(model, kw):
    """At a uniform T every cell's relaxation times and etaP are the
    constants times the factors: the isothermal correct() of the scaled
    model, to the last bits."""
    import ctypes as C
    from oracle import pyoracle
    from oracle.pyoracle import Oracle
    case = model_cavity(model, kw)
    m = case.model
    m.thermoLambda = ThermoFunction("Arrhenius", alpha=3000.0, T0=320.0)
    m.thermoLambda2 = ThermoFunction("WLF", c1=0.886, c2=101.6, T0=300.0)
    m.thermoEta = ThermoFunction("ArrheniusModified", alpha=0.015, T0=310.0)
    f0 = developed(case)
    T = 345.0
    shifted = Oracle(case, f0.copy())
    shifted.constitutive_correct(T=np.full(case.mesh.nCells, T))
    f = lambda fn: pyoracle.lib().or_thermo_factor(C.byref(fn.to_c()), T)
    scaled = copy.deepcopy(case)
    sm = scaled.model
    sm.lambda_ = m.lambda_ * f(m.thermoLambda)
    sm.lambdaR = m.lambdaR * f(m.thermoLambda2)
    sm.lambdaS = m.lambdaS * f(m.thermoLambda2)
    sm.etaP = m.etaP * f(m.thermoEta)
    iso = Oracle(scaled, f0.copy())
    iso.constitutive_correct()
    for name in ("theta", "tau", "eigVals", "taub"):
        assert rel(getattr(shifted.f, name), getattr(iso.f, name)) < 1e-15, name


def test_oracle_temperature_field_shifts_cell_by_cell():
    """A non-uniform temperature with only etaP shifted (thermoEta
    Arrhenius, thermoLambda Constant): the theta equation does not see etaP,
    so theta is the isothermal one to the last bit, and each cell's tau is
    the isothermal tau times that cell's factor."""
    from oracle.pyoracle import Oracle
    case = model_cavity("GiesekusLog", {"alpha": 0.1})
    fn = ThermoFunction("Arrhenius", alpha=2000.0, T0=300.0)
    case.model.thermoEta = fn
    f0 = developed(case)
    x = case.mesh.C[:, 0]
    T = np.where(x > np.median(x), 360.0, 300.0) + 5.0 * case.mesh.C[:, 1]
    hot = Oracle(case, f0.copy())
    hot.constitutive_correct(T=T)
    iso = Oracle(case, f0.copy())
    iso.constitutive_correct()
    assert np.array_equal(hot.f.theta, iso.f.theta)
    want = iso.f.tau * fn.factor(T)[:, None]
    assert rel(hot.f.tau, want) < 1e-14
    assert rel(hot.f.tau, iso.f.tau) > 0.1
