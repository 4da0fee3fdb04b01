"""The allocation-free red/black Ppe (wolfd2gpu_ppe_rbsor_noalloc) against
the context-based wolfd2gpu_ppe, through the C-ABI, on two calls in a row.

The entry point exists for callers that cannot call cudaMalloc (a driver
that has given all device memory to its own pool, or a solve loop that must
not reach the allocator): it takes device arrays the caller owns and keeps
its scratch in a fixed static device array.  The second call uses different
inputs, so state left in the shared scratch by the first call must not leak
into it.  The test allocates its own device buffers with torch; the entry
point itself allocates nothing."""
import numpy as np
import pytest

from wolfd2_gb300 import deck
from wolfd2_gb300.gpu import Solver, ppe_rbsor_noalloc, NOALLOC_MAX_POINTS, W2Error

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10


def _fields(case, seed):
    rng = np.random.default_rng(seed)
    shape = (case.nx + 2, case.ny + 2)
    x = np.linspace(0, 1, shape[0])[:, None]
    y = np.linspace(0, 1, shape[1])[None, :]
    out = []
    for _ in range(3):
        f = np.zeros(shape, order="F")
        for _ in range(4):
            k, l = rng.integers(1, 6, size=2)
            f += 0.05 * rng.normal() * np.sin(k * np.pi * x + rng.uniform(0, 6)) * np.cos(l * np.pi * y)
        out.append(np.asfortranarray(f))
    return out


def _device_metrics(torch, met):
    return {k: torch.from_numpy(np.ascontiguousarray(met[k].T)).cuda()
            for k in ("rau", "rgv", "xeu", "yeu", "xzv", "yzv")}


def _call(case, dm, du, dv, dp, prm, msorit, npsolver=5):
    return ppe_rbsor_noalloc(case.nx, case.ny, case.nx + 2, msorit, prm.dk, prm.sortol, prm.sorrel,
                             dm["rau"].data_ptr(), dm["rgv"].data_ptr(), dm["xeu"].data_ptr(),
                             dm["yeu"].data_ptr(), dm["xzv"].data_ptr(), dm["yzv"].data_ptr(),
                             du.data_ptr(), dv.data_ptr(), dp.data_ptr(), npsolver=npsolver)


@pytest.mark.parametrize("n, ny, npsolver", [(96, 72, 5), (97, 71, 5), (97, 71, 6)])
def test_noalloc_matches_context_ppe_twice(n, ny, npsolver):
    """Two calls in a row with different inputs, each equal bit for bit to
    the context Ppe with the same solver.  Odd nx leaves a colour's last
    column empty on alternate rows.  The second call must not change the
    device's free memory: the entry point allocates nothing."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    case = deck.cavity(n, 400.0, 0.002, solver="rb_sor", ny=ny)
    s = Solver(case.nx, case.ny, case.regions)
    met = s.grid_metric(case.x, case.y, want=True)

    def dev(a):  # Fortran (ld, ny+2) array -> device buffer with the same layout
        return torch.from_numpy(np.ascontiguousarray(a.T)).cuda()

    dm = _device_metrics(torch, met)
    prm = case.params
    for call, seed in enumerate((11, 12)):
        u, v, p = _fields(case, seed)
        s.VelBoundCond(u, v)
        s.PresBoundCond(p)
        p_ctx = p.copy(order="F")
        n_ctx = s.Ppe(True, npsolver, 400, prm.dk, prm.sortol, prm.sorrel, u, v, p_ctx)
        du, dv, dp = dev(u), dev(v), dev(p)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        n_na = _call(case, dm, du, dv, dp, prm, 400, npsolver)
        free1 = torch.cuda.mem_get_info()[0]
        if call == 1:
            assert free1 == free0, (free0, free1)
        p_na = np.asfortranarray(dp.cpu().numpy().T)
        assert n_na == n_ctx, (call, n_na, n_ctx)
        rel = float(np.max(np.abs(p_na - p_ctx)) / np.max(np.abs(p_ctx)))
        assert rel <= REL_TOL, (call, rel)
        assert np.array_equal(p_na, p_ctx), call


def test_noalloc_rejects_unsupported_arguments():
    """A curvilinear flag and a leading dimension shorter than a row are
    refused before anything is launched."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    a = buf.data_ptr()
    nx = ny = 33
    with pytest.raises(W2Error) as ei:
        ppe_rbsor_noalloc(nx, ny, nx + 2, 10, 1e-3, 1e-8, 1.0, a, a, a, a, a, a, a, a, a, lcartes=0)
    assert ei.value.code == 6
    with pytest.raises(W2Error) as ei:
        ppe_rbsor_noalloc(nx, ny, nx + 1, 10, 1e-3, 1e-8, 1.0, a, a, a, a, a, a, a, a, a)
    assert ei.value.code == 1
    with pytest.raises(W2Error) as ei:
        ppe_rbsor_noalloc(nx, ny, nx + 2, 10, 1e-3, 1e-8, 1.0, a, a, a, a, a, a, a, a, a, npsolver=1)
    assert ei.value.code == 6


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    nx = ny = 1200                                   # (nx+2)*(ny+2) > W2_NOALLOC_MAX_POINTS
    assert (nx + 2) * (ny + 2) > NOALLOC_MAX_POINTS
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    a = buf.data_ptr()
    with pytest.raises(W2Error) as ei:
        ppe_rbsor_noalloc(nx, ny, nx + 2, 10, 1e-3, 1e-8, 1.0, a, a, a, a, a, a, a, a, a)
    assert ei.value.code == 8
