"""The allocation-free pressure solve (aj_poisson_mg_static).

Some callers cannot allocate device memory for a call: hosts that own all
device memory through their own allocator, or loops that cannot take
cudaMalloc's synchronisation.  For them the library keeps the multigrid's
scratch in a device array of its own.  This test calls that entry point
through the C ABI, twice in a row with different inputs, and checks each
result against the ordinary workspace-based entry point (aj_poisson_mg, via
poisson_multigrid) within the suite's FP32 tolerance, and against the
reference's own float64 multigrid (golden fixtures).  It sits in a file that
pytest collects last, and needs nothing from the other tests."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _params(nx, ny, dx, v_cycles, dy=None):
    from aerojax_gb300.params import StepConfig
    from aerojax_gb300.solver import make_params
    return make_params(StepConfig(nx=nx, ny=ny, dx=dx, dy=dx if dy is None else dy, nu=1.0,
                                  variant="gui", v_cycles=v_cycles, mg_mode="parity"))


def _static_solve(L, prm, rhs, mask):
    import torch
    p = torch.full_like(rhs, float("nan"))
    stats = torch.zeros(64, dtype=torch.uint8, device=rhs.device)
    rc = L.aj_poisson_mg_static(ctypes.byref(prm), rhs.data_ptr(), mask.data_ptr(), p.data_ptr(),
                                stats.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, rc
    return p


@pytest.mark.parametrize("nx,ny", [(512, 96), (2048, 512)])
def test_static_matches_workspace_solver_twice(cuda_lib, nx, ny):
    """512x96, and 2048x512: exactly AJ_STATIC_MAX_CELLS cells, the largest
    layout the library's array must hold."""
    import torch
    import aerojax_gb300 as aj
    L = cuda_lib
    dx, vc = 1 / 64, 3
    assert nx * ny <= 1 << 20
    prm = _params(nx, ny, dx, vc)
    rng = np.random.default_rng(11)
    mask = torch.as_tensor((rng.random((nx, ny)) > 0.05).astype(np.float32), device="cuda")
    results = []
    for call in range(2):                      # two calls in a row, different inputs
        rhs = torch.as_tensor((10.0 * rng.standard_normal((nx, ny))).astype(np.float32),
                              device="cuda")
        p_static = _static_solve(L, prm, rhs, mask)
        p_ref = aj.poisson_multigrid(rhs, mask, dx, dx, v_cycles=vc)
        torch.cuda.synchronize()
        assert torch.isfinite(p_static).all()
        err = float((p_static - p_ref).abs().max() / p_ref.abs().max())
        assert err < TOL, (call, err)
        results.append(p_static.clone())
    assert not torch.equal(results[0], results[1])


@pytest.mark.parametrize("name", ["mg_64x32", "mg_128x48"])
def test_static_matches_reference_fixture(cuda_lib, name):
    """The same entry point against the reference's own multigrid run in
    float64 (the golden fixtures of tests/golden, collocated operator), two
    calls in a row, within the suite's FP32 tolerance."""
    import torch
    from conftest import golden
    g = golden(name)
    nx, ny = g["rhs"].shape
    prm = _params(nx, ny, float(g["dx"]), int(g["v_cycles"]), float(g["dy"]))
    rhs = torch.as_tensor(g["rhs"].astype(np.float32), device="cuda")
    mask = torch.as_tensor(g["mask"].astype(np.float32), device="cuda")
    ref = np.asarray(g["p"], np.float64)
    for call in range(2):
        p = _static_solve(cuda_lib, prm, rhs, mask)
        torch.cuda.synchronize()
        err = float(np.max(np.abs(p.double().cpu().numpy() - ref)) / np.max(np.abs(ref)))
        assert err < TOL, (call, err)


def test_static_rejects_oversized_grid(cuda_lib):
    import torch
    L = cuda_lib
    nx, ny = 4096, 512                          # 2 Mi cells > AJ_STATIC_MAX_CELLS
    prm = _params(nx, ny, 1 / 64, 1)
    x = torch.zeros(16, device="cuda")          # never touched: rejected on the host
    rc = L.aj_poisson_mg_static(ctypes.byref(prm), x.data_ptr(), x.data_ptr(), x.data_ptr(),
                                None, torch.cuda.current_stream().cuda_stream)
    assert rc == 7                              # AJ_ERR_WORKSPACE
