"""Beam statistics and beam edits through the C ABI, FP64 and FP32 beams,
against the reference's formulas evaluated with numpy on the same input.

Formulas (src/beam/src/beam.cpp, beam_kernel.cu): averages and sigmas over
loss == 0 are divided by num_particle - num_loss; emittances are
normalised by beta*gamma of particle 0's energy; the relative phase wraps
phi - phi_0 into [-pi, pi); CutBeam flags particles 1..n-1 strictly inside
(lo, hi) with 99999; ShiftVariable moves particles 1..n-1.
Tolerances: FP64 beams 1e-12 relative; FP32 beams 2e-6 relative (sizes,
emittances) and 2e-6 sigma (centroids)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
PREC = ("fp64", "fp32")
MASS = 939.294


def make_dist(n=50000, seed=3):
    rng = np.random.default_rng(seed)
    x = rng.normal(0.0, 0.002, n)
    xp = 0.3 * x / 0.002 * 1e-3 + rng.normal(0.0, 1e-3, n)
    y = rng.normal(1e-4, 0.0015, n)
    yp = rng.normal(0.0, 8e-4, n)
    phi = 123.4 + rng.normal(0.0, 0.2, n)
    w = 2.5 + rng.normal(0.0, 0.004, n) + 0.01 * (phi - 123.4)
    loss = np.where(rng.random(n) < 0.05, 7, 0).astype(np.uint32)
    loss[0] = 0
    for v in (x, xp, y, yp):  # set_distribution puts the reference particle on axis
        v[0] = 0.0
    return x, xp, y, yp, phi, w, loss


def rel_phase(phi, ref):
    tmp = phi - ref + np.pi
    sign = np.where(tmp < 0, -1.0, 1.0)
    return sign * (np.fmod(np.abs(tmp), 2 * np.pi) - np.pi)


def expected(x, xp, y, yp, phi, w, loss):
    a = loss == 0
    sv = a.sum()
    def avg(v):
        return v[a].sum() / sv
    def sig(v):
        return np.sqrt((v[a] ** 2).sum() / sv - avg(v) ** 2)
    def emit(u, up):
        mu, mup = avg(u), avg(up)
        cov = (u[a] * up[a]).sum() / sv - mu * mup
        return np.sqrt((sig(u) ** 2) * (sig(up) ** 2) - cov * cov)
    g1 = w[0] / MASS
    bg = np.sqrt(g1 * (g1 + 2.0))
    pr = rel_phase(phi, phi[0])
    return dict(x_avg=avg(x), x_sig=sig(x), y_avg=avg(y), y_sig=sig(y), w_avg=avg(w), w_sig=sig(w),
                phi_avg=avg(phi), x_emit=emit(x, xp) * bg, y_emit=emit(y, yp) * bg, z_emit=emit(pr, w),
                phi_r=pr)


def beam_from(prec, dist):
    from hpsim_gb300 import HPSim
    x, xp, y, yp, phi, w, loss = dist
    b = HPSim.Beam(mass=MASS, charge=-1.0, current=0.015, num=len(x), precision=prec)
    b.set_distribution(x, xp, y, yp, phi, w, loss, np.zeros_like(loss))
    return b


def tol(prec):
    return 1e-12 if prec == "fp64" else 2e-6


@pytest.mark.parametrize("prec", PREC)
def test_moments_and_emittances(prec):
    dist = make_dist()
    e = expected(*dist)
    b = beam_from(prec, dist)
    t = tol(prec)
    assert b.get_loss_num("t") == int(np.sum(dist[-1] != 0))
    for name, got, scale in (("x_avg", b.get_avg_x(), e["x_sig"]), ("y_avg", b.get_avg_y(), e["y_sig"]),
                             ("w_avg", b.get_avg_w(), e["w_sig"]), ("phi_avg", b.get_avg_phi(), 0.2)):
        assert abs(got - e[name]) <= t * scale + 1e-12 * abs(e[name]), (name, got, e[name])
    # sigma = sqrt(<v^2> - <v>^2) loses (<v>/sigma)^2 ulps to cancellation in
    # FP64 (the reference's formula); FP32 beams sum offsets and do not
    cw = 1e-15 * (e["w_avg"] / e["w_sig"]) ** 2 if prec == "fp64" else 0.0
    for name, got, c in (("x_sig", b.get_sig_x(), 0.0), ("y_sig", b.get_sig_y(), 0.0), ("w_sig", b.get_sig_w(), cw),
                         ("x_emit", b.get_emittance_x(), 0.0), ("y_emit", b.get_emittance_y(), 0.0),
                         ("z_emit", b.get_emittance_z(), cw)):
        assert abs(got - e[name]) <= (t + c) * abs(e[name]), (name, got, e[name])


@pytest.mark.parametrize("prec", PREC)
def test_coordinates_round_trip(prec):
    dist = make_dist(n=4096)
    b = beam_from(prec, dist)
    names = ("x", "xp", "y", "yp", "phi", "w")
    for k, v in zip(names, dist[:6]):
        got = b._coord(k)
        want = v.copy()
        if prec == "fp64":
            assert np.array_equal(got, want), k
        else:
            anchor = v[0] if k in ("phi", "w") else 0.0
            assert np.allclose(got - anchor, (want - anchor).astype(np.float32), rtol=0, atol=1e-7 * np.abs(want - anchor).max()), k
    assert b.get_ref_w() == dist[5][0]
    assert b.get_ref_phi() == dist[4][0]
    pr = b.get_phi("all", "relative")
    assert np.allclose(pr, expected(*dist)["phi_r"], rtol=0, atol=1e-14 if prec == "fp64" else 1e-6)


@pytest.mark.parametrize("prec", PREC)
def test_cut_translate_and_reference_edits(prec):
    dist = make_dist(n=8192)
    x, xp, y, yp, phi, w, loss = dist
    b = beam_from(prec, dist)
    lo, hi = -0.001, 0.0005
    b.apply_cut("x", lo, hi)
    want = loss.copy()
    sel = (np.arange(len(x)) > 0) & (loss == 0) & (x > lo) & (x < hi)
    want[sel] = 99999
    assert np.array_equal(b.get_losses("t"), want)
    b.translate("w", 0.01)
    w2 = b._coord("w")
    assert w2[0] == w[0]
    assert np.allclose(w2[1:], w[1:] + 0.01, rtol=0, atol=1e-14 if prec == "fp64" else 2e-6)
    b.set_ref_w(2.6)
    b.set_ref_phi(124.0)
    assert b.get_ref_w() == 2.6
    assert b.get_ref_phi() == 124.0
    w3 = b._coord("w")
    assert np.allclose(w3[1:], w2[1:], rtol=0, atol=1e-14 if prec == "fp64" else 2e-6)


@pytest.mark.parametrize("prec", PREC)
def test_monitor_record(prec):
    dist = make_dist()
    e = expected(*dist)
    b = beam_from(prec, dist)
    m = b.monitor()
    t = tol(prec)
    assert m[0] == np.sum(dist[-1] == 0)
    assert abs(m[6] - e["x_emit"]) <= t * e["x_emit"]
    assert abs(m[11] - e["y_emit"]) <= t * e["y_emit"]
    cw = 1e-15 * (e["w_avg"] / e["w_sig"]) ** 2 if prec == "fp64" else 0.0
    assert abs(m[16] - e["z_emit"]) <= (t + cw) * e["z_emit"]
    assert abs(m[14] - e["w_avg"]) <= t * e["w_sig"] + 1e-12 * e["w_avg"]
