"""The backward kernel behind torch.autograd.Function, against the FP64
reference gradient (tests/test_oracle.py pins it to central differences) and
against FP64 central differences of the GPU's own f64 forward.

Tolerances: f64 gradients 1e-9 relative to max(|g|, 1); f32 gradients 2e-4
relative to the gradient's largest entry (atomic f32 accumulation over many
pairs).  Excluded from comparisons: each PCF's last value (its rectangle runs
to numeric_limits<T>::max()) only in the finite-difference check.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def native():
    from stablebear_gb300 import build
    build.build()


KINDS = [("l2_kernel", 2, 2, 1.0), ("l2", 1, 1, 2.0), ("l1", 0, 1, 1.0)]


def _grad_gpu(pts, off, kind, w):
    import torch
    from stablebear_gb300 import autograd as ag
    P = torch.tensor(pts, device="cuda", requires_grad=True)
    O = torch.tensor(off.astype(np.int64), device="cuda")
    M = ag.l2_kernel(P, O) if kind == "l2_kernel" else ag.pdist(P, O, p=2 if kind == "l2" else 1)
    loss = (torch.tensor(w, device="cuda", dtype=P.dtype) * M).sum()
    loss.backward()
    return P.grad.cpu().numpy().astype(np.float64), M.detach().cpu().numpy()


@pytest.mark.parametrize("kind,op,mode,p", KINDS)
def test_backward_f64_matches_reference_gradient(kind, op, mode, p):
    from stablebear_gb300 import synthetic
    from oracle import oracle as orc
    from tests.test_oracle import oracle_gradient
    pts, off = synthetic.gaussian(45, synthetic.uniform_lengths(1, 30), np.float64, seed=7)
    n = len(off) - 1
    cnt = n * (n + 1) // 2 if mode == 2 else n * (n - 1) // 2
    w = np.random.default_rng(2).standard_normal(cnt)
    g, M = _grad_gpu(pts, off, kind, w)
    ref = oracle_gradient(pts, off, op, mode, w, M if op == 1 else None)
    scale = np.maximum(np.abs(ref), 1.0)
    assert np.max(np.abs(g - ref) / scale) <= 1e-9


@pytest.mark.parametrize("kind,op,mode,p", KINDS)
def test_backward_f32_close_to_fp64_gradient(kind, op, mode, p):
    from stablebear_gb300 import synthetic
    from tests.test_oracle import oracle_gradient
    pts, off = synthetic.differentiation(300, seed=4)
    n = len(off) - 1
    cnt = n * (n + 1) // 2 if mode == 2 else n * (n - 1) // 2
    w = np.random.default_rng(3).standard_normal(cnt)
    g, M = _grad_gpu(pts, off, kind, w.astype(np.float32))
    ref = oracle_gradient(pts.astype(np.float64), off, op, mode, w.astype(np.float32).astype(np.float64),
                          M.astype(np.float64) if op == 1 else None)
    # compare away from each PCF's last value (rectangle to FLT_MAX) and t_0
    mask = np.ones(pts.shape, bool)
    mask[(off[1:] - 1).astype(int), 1] = False
    mask[off[:-1].astype(int), 0] = False
    err = np.abs(g - ref)[mask].max() / np.abs(ref[mask]).max()
    assert err <= 2e-4


def test_backward_f64_matches_central_differences_of_gpu_forward():
    import torch
    from stablebear_gb300 import autograd as ag, synthetic
    pts, off = synthetic.gaussian(20, synthetic.uniform_lengths(2, 12), np.float64, seed=9)
    n = len(off) - 1
    G = np.random.default_rng(5).standard_normal((n, n))
    G = G + G.T  # random symmetric upstream matrix
    O = torch.tensor(off.astype(np.int64), device="cuda")

    def loss(p_np, grad=False):
        P = torch.tensor(p_np, device="cuda", requires_grad=grad)
        K = ag.condensed_to_dense(ag.l2_kernel(P, O), n, diagonal=True)
        D = ag.condensed_to_dense(ag.pdist(P, O, p=2), n, diagonal=False)
        L = (torch.tensor(G, device="cuda") * (K + D)).sum()
        if grad:
            L.backward()
            return float(L), P.grad.cpu().numpy()
        return float(L)

    _, g = loss(pts, grad=True)
    starts = set(int(x) for x in off[:-1])
    lasts = set(int(x) - 1 for x in off[1:])
    eps = 1e-6
    checked = 0
    for k in range(0, len(pts), 3):
        for c in (0, 1):
            if (c == 0 and k in starts) or (c == 1 and k in lasts):
                continue
            q = pts.copy()
            q[k, c] += eps
            a = loss(q)
            q[k, c] -= 2 * eps
            b = loss(q)
            fd = (a - b) / (2 * eps)
            assert abs(fd - g[k, c]) <= 1e-6 * max(1.0, abs(fd)), (k, c, fd, g[k, c])
            checked += 1
    assert checked >= 20


def test_forward_of_autograd_path_equals_pdist():
    import torch
    import stablebear_gb300 as sb
    from stablebear_gb300 import autograd as ag, synthetic
    pts, off = synthetic.differentiation(200, seed=1)
    P = torch.tensor(pts, device="cuda")
    O = torch.tensor(off.astype(np.int64), device="cuda")
    X = sb.PcfArray.from_csr(pts, off)
    np.testing.assert_allclose(ag.pdist(P, O, p=2).cpu().numpy(), sb.pdist(X, p=2).data, rtol=1e-5)
    np.testing.assert_allclose(ag.l2_kernel(P, O).cpu().numpy(), sb.l2_kernel(X).data, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("lengths", [(16, 500), (520, 620), (700, 900)])
def test_backward_f32_walk_shapes(lengths):
    """The float32 backward stages the item's columns in shared memory with
    windows of 12 row elements while PCFs are short enough (up to about 515
    breakpoints), with windows of 8 a little beyond, and reads them through
    L1 with windows of 16 above that: each shape against the FP64 reference
    gradient, L2 kernel and L1 distance."""
    from stablebear_gb300 import synthetic
    from tests.test_oracle import oracle_gradient
    lo, hi = lengths
    pts, off = synthetic.gaussian(70, synthetic.uniform_lengths(lo, hi), np.float32, seed=lo)
    n = len(off) - 1
    mask = np.ones(pts.shape, bool)
    mask[(off[1:] - 1).astype(int), 1] = False
    mask[off[:-1].astype(int), 0] = False
    for kind, op, mode in (("l2_kernel", 2, 2), ("l1", 0, 1)):
        cnt = n * (n + 1) // 2 if mode == 2 else n * (n - 1) // 2
        w = np.random.default_rng(lo + mode).standard_normal(cnt).astype(np.float32)
        g, M = _grad_gpu(pts, off, kind, w)
        ref = oracle_gradient(pts.astype(np.float64), off, op, mode, w.astype(np.float64), None)
        err = np.abs(g - ref)[mask].max() / np.abs(ref[mask]).max()
        assert err <= 2e-4, (kind, lengths, err)


def _torch_expand(c, n, diagonal):
    import torch
    k = 0 if diagonal else -1
    r, s = torch.tril_indices(n, n, offset=k, device=c.device)
    dense = torch.zeros(n, n, dtype=c.dtype, device=c.device)
    dense = dense.index_put((r, s), c)
    return dense + torch.tril(dense, -1).transpose(0, 1)


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("diagonal", [True, False])
@pytest.mark.parametrize("n", [1, 2, 65, 300])
def test_condensed_to_dense_and_its_gradient(dtype, diagonal, n):
    """The native expansion (sbg_condensed_to_dense_device) and its gradient
    (sbg_dense_fold_to_condensed_device) against the same expansion written
    with torch indexing ops: both bit for bit (the gradient of an
    off-diagonal entry is G_ij + G_ji either way)."""
    import torch
    from stablebear_gb300 import autograd as ag
    dt = getattr(torch, dtype)
    cnt = n * (n + 1) // 2 if diagonal else n * (n - 1) // 2
    gen = torch.Generator("cuda").manual_seed(n + (7 if diagonal else 0))
    c = torch.randn(cnt, dtype=dt, device="cuda", generator=gen).requires_grad_(True)
    G = torch.randn(n, n, dtype=dt, device="cuda", generator=gen)
    c2 = c.detach().clone().requires_grad_(True)
    D = ag.condensed_to_dense(c, n, diagonal)
    (G * D).sum().backward()
    D2 = _torch_expand(c2, n, diagonal)
    (G * D2).sum().backward()
    assert torch.equal(D, D2)
    assert torch.equal(c.grad, c2.grad)


def test_given_max_points_changes_nothing():
    """A caller that knows the longest PCF passes max_points and skips the
    read-back: the same forward result bit for bit, and the same gradient up
    to the order of its atomic float32 additions."""
    import torch
    from stablebear_gb300 import autograd as ag, synthetic
    pts, off = synthetic.differentiation(160, seed=5)
    lmax = int(np.diff(off.astype(np.int64)).max())
    O = torch.tensor(off.astype(np.int64), device="cuda")
    out = []
    for mp in (None, lmax):
        P = torch.tensor(pts, device="cuda", requires_grad=True)
        M = ag.l2_kernel(P, O, max_points=mp)
        (M * M).sum().backward()
        out.append((M.detach().clone(), P.grad.clone()))
    assert torch.equal(out[0][0], out[1][0])
    g0, g1 = out[0][1], out[1][1]
    assert float((g0 - g1).abs().max()) <= 1e-5 * float(g0.abs().max())
