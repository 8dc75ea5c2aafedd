"""Temperature-dependent parameters on the GPU (rt_set_temperature): the
constitutiveEq::correct() of a non-isothermal solver (rheoHeatFoam.C:144,189)
against the FP64 oracle's, every Log model with its thermoFunctions at a
temperature field that varies from cell to cell."""
import numpy as np
import pytest

from rheotool_gb300 import abi
from rheotool_gb300.case import ThermoFunction, cavity_case

from test_gpu_parity import MODELS, flow_state, model_cavity, multimode_case, recon, rel

pytestmark = pytest.mark.gpu

# one set of functions per model, every type used somewhere
FUNCS = [
    (ThermoFunction("Arrhenius", alpha=3000.0, T0=320.0), ThermoFunction("WLF", c1=0.886, c2=101.6, T0=300.0),
     ThermoFunction("ArrheniusModified", alpha=0.015, T0=310.0)),
    (ThermoFunction("WLF", c1=0.886, c2=101.6, T0=300.0), ThermoFunction("Constant"),
     ThermoFunction("VFT", A=500.0, B=-2.5, T0=150.0)),
    (ThermoFunction("VFT", A=100.0, B=-0.5, T0=200.0), ThermoFunction("Arrhenius", alpha=2000.0, T0=330.0),
     ThermoFunction("Arrhenius", alpha=2500.0, T0=330.0)),
]


def temperature(case):
    """300 K .. 360 K across the cavity, with a bump in the middle."""
    x, y = case.mesh.C[:, 0], case.mesh.C[:, 1]
    return 300.0 + 60.0 * x + 15.0 * np.exp(-40.0 * ((x - 0.5) ** 2 + (y - 0.5) ** 2))


@pytest.mark.parametrize("i", range(len(MODELS)))
def test_constitutive_correct_with_temperature_matches_oracle(ctx, i):
    from oracle.pyoracle import Oracle
    model, kw = MODELS[i]
    case = model_cavity(model, kw)
    m = case.model
    m.thermoLambda, m.thermoLambda2, m.thermoEta = FUNCS[i % len(FUNCS)]
    f0 = flow_state(case)
    T = temperature(case)
    ctx.setup_case(case, f0)
    try:
        ctx.set_temperature(T)
        perf_g = ctx.constitutive_correct()
        got = ctx.fields()
    finally:
        ctx.set_temperature(None)
    o = Oracle(case, f0.copy())
    perf_o = o.constitutive_correct(T=T)
    for k in range(6):
        assert perf_g[k].nIterations == perf_o[k].nIterations
    for name in ("theta", "tau", "eigVals", "taub"):
        assert rel(getattr(got, name), getattr(o.f, name)) < 1e-11, name
    assert rel(recon(got.eigVals, got.eigVecs), recon(o.f.eigVals, o.f.eigVecs)) < 1e-11
    # the shifts act: the isothermal correct() gives another tau
    iso = Oracle(case, f0.copy())
    iso.constitutive_correct()
    assert rel(got.tau, iso.f.tau) > 1e-3


def test_multimode_constitutive_correct_with_temperature(ctx):
    """Each mode with its own thermoFunctions."""
    from oracle.pyoracle import Oracle
    case = multimode_case(cavity_case(10, model="Oldroyd-BLog"))
    for mm, (fl, f2, fe) in zip(case.models, FUNCS):
        mm.thermoLambda, mm.thermoLambda2, mm.thermoEta = fl, f2, fe
    o = Oracle(case)
    o.step(2)
    f0 = o.f.copy()
    T = temperature(case)
    o.constitutive_correct(T=T)
    ctx.setup_case(case, f0)
    try:
        ctx.set_temperature(T)
        ctx.constitutive_correct()
        got = ctx.fields()
    finally:
        ctx.set_temperature(None)
    for k in range(3):
        for name in ("theta", "tau"):
            assert rel(getattr(got.modes[k], name), getattr(o.f.modes[k], name)) < 1e-11, (k, name)
    assert rel(got.tau, o.f.tau) < 1e-11


def test_mixed_constitutive_correct_with_temperature(ctx):
    """The mixed form's FP32 constitutive update takes the same shifts:
    within the mixed bar (1e-6) of the FP64 oracle."""
    from oracle.pyoracle import Oracle
    case = model_cavity("GiesekusLog", {"alpha": 0.1})
    case.model.thermoLambda, case.model.thermoLambda2, case.model.thermoEta = FUNCS[0]
    f0 = flow_state(case)
    T = temperature(case)
    case.precision = abi.RT_PREC_MIXED
    ctx.setup_case(case, f0)
    try:
        ctx.set_temperature(T)
        ctx.constitutive_correct()
        got = ctx.fields()
    finally:
        ctx.set_temperature(None)
        case.precision = abi.RT_PREC_FP64
    o = Oracle(case, f0.copy())
    o.constitutive_correct(T=T)
    for name in ("theta", "tau"):
        assert rel(getattr(got, name), getattr(o.f, name)) < 1e-6, name


def test_temperature_off_is_the_isothermal_case(ctx):
    """rt_set_temperature(NULL) returns to the isothermal correct(), bit for
    bit; a new case setup clears the temperature too."""
    case = model_cavity("GiesekusLog", {"alpha": 0.1})
    case.model.thermoLambda, case.model.thermoLambda2, case.model.thermoEta = FUNCS[0]
    f0 = flow_state(case)
    ctx.setup_case(case, f0)
    ctx.constitutive_correct()
    plain = ctx.fields()
    ctx.setup_case(case, f0)
    ctx.set_temperature(temperature(case))
    ctx.set_temperature(None)
    ctx.constitutive_correct()
    off = ctx.fields()
    ctx.setup_case(case, f0)
    ctx.set_temperature(temperature(case))
    ctx.setup_case(case, f0)
    ctx.constitutive_correct()
    again = ctx.fields()
    for name in ("theta", "tau"):
        assert np.array_equal(getattr(plain, name), getattr(off, name)), name
        assert np.array_equal(getattr(plain, name), getattr(again, name)), name


def test_temperature_errors(ctx):
    """A temperature outside a function's domain, an unknown type and a time
    step with a temperature set are refused with RT_EINVAL; the context
    stays usable."""
    from rheotool_gb300.runtime import RheoGpuError
    case = model_cavity("Oldroyd-BLog", {})
    case.model.thermoLambda = ThermoFunction("Arrhenius", alpha=3000.0, T0=320.0)
    ctx.setup_case(case)
    T = temperature(case)
    bad = T.copy()
    bad[3] = -1.0
    with pytest.raises(RheoGpuError) as e:
        ctx.set_temperature(bad)
    assert e.value.status == abi.RT_EINVAL
    case.model.thermoEta = ThermoFunction("VFT", A=500.0, B=-2.5, T0=float(T[5]))
    with pytest.raises(RheoGpuError) as e:
        ctx.set_temperature(T)
    assert e.value.status == abi.RT_EINVAL
    case.model.thermoEta = ThermoFunction("Constant")
    descs = case.thermo_descs()
    descs[0].lambda2.type = 9
    st = ctx.lib.rt_set_temperature(ctx._ctx, descs, abi.dptr(np.ascontiguousarray(T)))
    assert st == abi.RT_EINVAL
    ctx.set_temperature(T)
    try:
        with pytest.raises(RheoGpuError) as e:
            ctx.step(1)
        assert e.value.status == abi.RT_EINVAL
    finally:
        ctx.set_temperature(None)
    ctx.step(1)
