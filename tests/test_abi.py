"""The C-ABI library loads without a GPU, exports every symbol the header
declares, agrees with the header on struct layout, and its host-side checks
mirror the reference's trace-time errors.  No compute calls.  CPU only."""
import ctypes
import os
import subprocess

import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def L():
    from aerojax_gb300 import build, _lib
    build.build()
    return _lib.lib()


def test_exports_every_header_symbol(L):
    from aerojax_gb300 import _lib
    names = _lib.header_symbols()
    assert len(names) >= 10
    for n in names:
        assert hasattr(L, n), f"{n} declared in include/aerojax_gb300.h but not exported"
    assert L.aj_version() == 100


def test_struct_layout_matches_header(tmp_path):
    from aerojax_gb300 import _lib
    src = tmp_path / "sz.c"
    src.write_text('#include "aerojax_gb300.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                   'int main(){printf("%zu %zu %zu %zu\\n", sizeof(AjStepParams), sizeof(AjStats),'
                   ' offsetof(AjStepParams, dx), offsetof(AjStepParams, les_delta));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)]).decode().split()
    P = _lib.AjStepParams
    assert int(out[0]) == ctypes.sizeof(P)
    assert int(out[1]) == ctypes.sizeof(_lib.AjStats)
    assert int(out[2]) == P.dx.offset
    assert int(out[3]) == P.les_delta.offset


def _params(**kw):
    from aerojax_gb300.params import StepConfig
    from aerojax_gb300.solver import make_params
    base = dict(nx=512, ny=96, dx=1 / 64, dy=1 / 64, nu=1e-3, v_cycles=3, dt=1e-3)
    base.update(kw)
    return make_params(StepConfig(**base))


@pytest.mark.parametrize("shape,status", [((512, 96), 0), ((2048, 512), 0), ((100, 64), 1),
                                          ((64, 40), 1), ((32, 16), 1)])
def test_parity_shape_rule(L, shape, status):
    """aj_check_params returns AJ_ERR_SHAPE exactly where poisson_multigrid
    raises ValueError (multigrid_solver.py:96-106)."""
    p = _params(nx=shape[0], ny=shape[1])
    assert L.aj_check_params(ctypes.byref(p)) == status
    if status == 0:
        assert L.aj_workspace_size(ctypes.byref(p)) > 0
    else:
        assert L.aj_workspace_size(ctypes.byref(p)) == 0


def test_param_errors(L):
    assert L.aj_check_params(ctypes.byref(_params(dx=0.0))) == 2
    # step_pure cannot run on the MAC grid (step.py:348 shape broadcast)
    assert L.aj_check_params(ctypes.byref(_params(grid_type="mac", variant="pure"))) == 2
    assert L.aj_check_params(ctypes.byref(_params(grid_type="mac", variant="gui"))) == 0
    assert L.aj_check_params(ctypes.byref(_params(mg_mode="converge", mg_rtol=0.0))) == 2
    assert L.aj_check_params(ctypes.byref(_params(mg_mode="converge"))) == 0
    # AJ_WARM_EXTRAPOLATE exists for the converging solve only
    assert L.aj_check_params(ctypes.byref(_params(mg_mode="converge",
                                                  warm_start="extrapolate"))) == 0
    assert L.aj_check_params(ctypes.byref(_params(warm_start="extrapolate"))) == 2
    p = _params(mg_mode="converge")
    p.warm_start = 3
    assert L.aj_check_params(ctypes.byref(p)) == 2


def test_extrapolation_history_in_workspace(L):
    """The extrapolation warm start keeps two double-FP32 solutions (16 bytes
    per cell) in the workspace."""
    a = L.aj_workspace_size(ctypes.byref(_params(mg_mode="converge", warm_start=True)))
    b = L.aj_workspace_size(ctypes.byref(_params(mg_mode="converge", warm_start="extrapolate")))
    assert b - a >= 16 * 512 * 96


def test_workspace_grows_with_grid(L):
    a = L.aj_workspace_size(ctypes.byref(_params(nx=512, ny=96)))
    b = L.aj_workspace_size(ctypes.byref(_params(nx=2048, ny=512)))
    assert b > 16 * a > 0


def test_converge_depth_rule_matches_oracle(L):
    """The CUDA converging hierarchy and the oracle's coarsen the same way."""
    from oracle import ref_np as R
    for shape in [(2048, 512), (512, 96), (768, 192), (1024, 256), (256, 64), (64, 32)]:
        assert R.mg_depth(*shape) >= 1
        p = _params(nx=shape[0], ny=shape[1], mg_mode="converge")
        assert L.aj_check_params(ctypes.byref(p)) == 0


def test_no_cpu_fallback_without_library(monkeypatch, tmp_path):
    """A missing library is an error, never a silent fallback."""
    from aerojax_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.lib()


def test_step_vjp_covers_the_rollout_configuration_only(L):
    """aj_step_vjp's host checks: the collocated von Karman step_pure, or the
    GUI step without LES, with upwind RK3/RK2, a fixed dt and the parity
    V-cycle; anything else gets no workspace size and no kernel count
    (aj_step_vjp itself returns AJ_ERR_PARAM)."""
    from dataclasses import replace
    from aerojax_gb300.adjoint import _config
    from aerojax_gb300.solver import make_params
    base = _config(128, 64, 0.05, 0.05, 0.02, 1.0, 4e-3, True)
    for ok in (base, replace(base, fast_mode=True), replace(base, v_cycles=3)):
        p = make_params(ok)
        assert L.aj_step_vjp_workspace_size(ctypes.byref(p)) > 0
        assert L.aj_step_vjp_kernel_count(ctypes.byref(p)) > 0
    gui = replace(base, variant="gui", nu_hyper_ratio=0.05, slip_walls=False)
    for ok in (gui, replace(gui, fast_mode=True, nu_hyper_ratio=0.0)):
        assert L.aj_step_vjp_workspace_size(ctypes.byref(make_params(ok))) > 0
    for bad in (replace(base, grid_type="mac", variant="gui"),
                replace(gui, use_les=True, les_model="smagorinsky"),
                replace(base, mg_mode="converge"), replace(base, cfl_dt=True),
                replace(base, advection_scheme="weno5"), replace(base, warm_start=True)):
        p = make_params(bad)
        assert L.aj_step_vjp_workspace_size(ctypes.byref(p)) == 0
        assert L.aj_step_vjp_kernel_count(ctypes.byref(p)) == -1
    # the reversed V-cycles and the recomputed stages are counted
    k1 = L.aj_step_vjp_kernel_count(ctypes.byref(make_params(base)))
    k3 = L.aj_step_vjp_kernel_count(ctypes.byref(make_params(replace(base, v_cycles=3))))
    assert k3 > k1
