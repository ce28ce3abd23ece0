"""The surrogate layers' oracle (oracle/nn_oracle.py): its backward pass
against central finite differences of its forward pass, for every layer
shape the network uses (stride 2, 2x upsampling), and BF16 rounding."""
import numpy as np
import pytest

from oracle import nn_oracle as N


@pytest.mark.parametrize("stride,up,relu", [(1, 1, 1), (2, 1, 1), (1, 2, 1), (1, 1, 0)])
def test_backward_matches_finite_differences(stride, up, relu):
    rng = np.random.default_rng(stride * 10 + up + relu)
    B, Ci, Co, H, W = 2, 3, 4, 8, 6
    x = rng.normal(size=(B, Ci, H, W))
    w = rng.normal(size=(Co, Ci, 3, 3))
    b = rng.normal(size=Co)
    z, y = N.conv_forward(x, w, b, stride, up, relu)
    g = rng.normal(size=y.shape)                # loss = sum(g * y)
    dz, dx, dw, db = N.conv_backward(x, w, y, relu, g, stride, up)
    loss = lambda x_, w_, b_: float((g * N.conv_forward(x_, w_, b_, stride, up, relu)[1]).sum())  # noqa: E731
    eps = 1e-6
    for arr, grad in ((w, dw), (b, db), (x, dx)):
        flat = arr.reshape(-1)
        for k in rng.choice(flat.size, min(12, flat.size), replace=False):
            old = flat[k]
            flat[k] = old + eps
            lp = loss(x, w, b)
            flat[k] = old - eps
            lm = loss(x, w, b)
            flat[k] = old
            assert abs((lp - lm) / (2 * eps) - grad.reshape(-1)[k]) < 1e-5 * max(1.0, abs(grad.reshape(-1)[k]))


def test_gmean_backward_is_the_adjoint():
    rng = np.random.default_rng(3)
    y, d = rng.normal(size=(2, 3, 4, 5)), rng.normal(size=(2, 3, 4, 5))
    assert np.isclose((N.gmean_forward(y) * d).sum(), (y * N.gmean_backward(d)).sum())


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e38], np.float32)
    r = N.bf16_round(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7 and r[3] == -2.5


def test_network_backward_matches_finite_differences():
    """The composed network (skip additions, plane-mean broadcast, strided
    and upsampling layers) of the surrogate's layer table, at reduced width."""
    from hpsim_gb300.surrogate import ARCH, GMEAN_AFTER, SKIP
    rng = np.random.default_rng(5)
    arch = [(min(ci, 3) if l else ci, min(co, 3) if l < len(ARCH) - 1 else co, s, u, r)
            for l, (ci, co, s, u, r) in enumerate(ARCH)]
    ws = [rng.normal(size=(co, ci, 3, 3)) / np.sqrt(9 * ci) for ci, co, *_ in arch]
    bs = [rng.normal(size=co) * 0.1 for _, co, *_ in arch]
    x = rng.normal(size=(2, arch[0][0], 32, 16))
    fwd = N.net_forward(x, ws, bs, arch, GMEAN_AFTER, SKIP)
    g = rng.normal(size=fwd[2][-1].shape)
    dws, dbs = N.net_backward(fwd, ws, arch, GMEAN_AFTER, SKIP, g)

    def loss():
        return float((g * N.net_forward(x, ws, bs, arch, GMEAN_AFTER, SKIP)[2][-1]).sum())

    eps = 1e-6
    for l in (0, 2, 4, 5, 8, 9):
        for arr, grad in ((ws[l], dws[l]), (bs[l], dbs[l])):
            flat = arr.reshape(-1)
            for k in rng.choice(flat.size, min(4, flat.size), replace=False):
                old = flat[k]
                flat[k] = old + eps
                lp = loss()
                flat[k] = old - eps
                lm = loss()
                flat[k] = old
                ref = grad.reshape(-1)[k]
                assert abs((lp - lm) / (2 * eps) - ref) < 1e-5 * max(1.0, abs(ref)), (l, k)
