"""Learned SCHEFF field surrogate: a small convolutional encoder-decoder that
maps the deposited r-z charge of a kick to (E_r, E_z) on the mesh, trained on
snapshots of the plain SCHEFF solver by this project's own forward and
backward kernels (csrc/nn.cu; PyTorch only holds the device buffers).

Scale-free form.  With every length in units of dr and the cell aspect
a = dz*gamma/dr fixed, the Green's function scales as 1/dr^2 and the field as
c1 * sum(q) / dr^2 (c1 = 5721.67 I f / (f_MHz 1e6 N m), the solver's
Green's-table scale).  The network sees q / sum(q) (times nr*nz) and log a,
and predicts E dr dz gamma / (c1 sum(q)) (the scale-free field times a) times
a fixed scale, on the nz x nr interior field points (zp < nz, rp < nr).

Network: a U-shaped encoder-decoder of 3x3 convolutions.  Four stride-2
layers take the 128 x 32 mesh down to 8 x 2 (channels 32-64-128-128-128), so
the coarsest layer sees the whole bunch (the Coulomb field is long-range),
and its channels get their plane mean added; four nearest-2x upsampling
layers come back up (128-128-64-32), each adding the encoder activation of
the same resolution (skip connections keep the near field), and a last layer
gives (E_r, E_z).  About 0.8 M parameters.  BF16 activations and weights in
the forward pass, FP32 sums, FP32 master weights and Adam.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from ._capi import call

# (c_in, c_out, stride, up, relu); the plane-mean broadcast follows layer
# GMEAN_AFTER; SKIP[l] = the layer whose output is added to layer l's
ARCH = [(2, 32, 1, 1, 1), (32, 64, 2, 1, 1), (64, 128, 2, 1, 1), (128, 128, 2, 1, 1), (128, 128, 2, 1, 1),
        (128, 128, 1, 2, 1), (128, 128, 1, 2, 1), (128, 64, 1, 2, 1), (64, 32, 1, 2, 1), (32, 2, 1, 1, 0)]
GMEAN_AFTER = 4
SKIP = {5: 3, 6: 2, 7: 1, 8: 0}
NZ, NR = 128, 32


def _p(t):
    return C.c_void_p(t.data_ptr())


def layer_shapes(batch, h=NZ, w=NR):
    """dims (int32[7]) of each layer for a batch of h x w inputs."""
    out = []
    for ci, co, s, u, _ in ARCH:
        out.append(np.array([batch, ci, co, h, w, s, u], dtype=np.int32))
        h, w = (h * u - 1) // s + 1, (w * u - 1) // s + 1
    return out


class Network:
    """Weights, Adam state and the forward / backward passes of the
    surrogate on the GPU (torch tensors as device buffers)."""

    def __init__(self, seed=0, device="cuda"):
        import torch
        self.torch, self.device = torch, device
        rng = np.random.default_rng(seed)
        self.w, self.b = [], []
        for ci, co, *_ in ARCH:
            std = math.sqrt(2.0 / (ci * 9))  # He initialisation
            self.w.append(torch.tensor(rng.normal(0.0, std, (co, ci, 3, 3)), dtype=torch.float32, device=device))
            self.b.append(torch.zeros(co, dtype=torch.float32, device=device))
        self.wb = [w.to(torch.bfloat16) for w in self.w]
        self.m = [torch.zeros_like(t) for t in self.w + self.b]
        self.v = [torch.zeros_like(t) for t in self.w + self.b]
        self.step_count = 0
        self.out_scale = 1.0
        # forward layers of batches of two or more on the tensor cores (the
        # layer shapes the kernel takes): measured 1.9x faster than the
        # CUDA-core layers over the whole network at batch 8, 2.8x at 32,
        # and no faster at batch 1
        self.tensor_cores = True
        self._tiles = {}      # (layer, dims) -> (device tiles, weight version)
        self._wver = 0        # bumped whenever the BF16 weights change
        self._tc_err = torch.zeros(1, dtype=torch.int32, device=device)

    # ---- state -------------------------------------------------------------
    def state(self):
        return {**{f"w{i}": w.cpu().numpy() for i, w in enumerate(self.w)},
                **{f"b{i}": b.cpu().numpy() for i, b in enumerate(self.b)},
                "out_scale": np.float64(self.out_scale)}

    def load(self, st):
        torch = self.torch
        self.w = [torch.tensor(st[f"w{i}"], dtype=torch.float32, device=self.device) for i in range(len(ARCH))]
        self.b = [torch.tensor(st[f"b{i}"], dtype=torch.float32, device=self.device) for i in range(len(ARCH))]
        self.wb = [w.to(torch.bfloat16) for w in self.w]
        self.out_scale = float(st["out_scale"])
        self._wver += 1

    def save(self, path):
        np.savez(path, **self.state())

    # ---- passes ------------------------------------------------------------
    def _layer_tiles(self, li, dims):
        """The tensor-core kernel's weight tiles of layer li at this shape
        (laid out again after the weights changed); None when the kernel
        does not take the shape."""
        key = (li, tuple(int(v) for v in dims))
        hit = self._tiles.get(key)
        if hit is not None and hit[1] == self._wver:
            return hit[0]
        dp = dims.ctypes.data_as(C.POINTER(C.c_int))
        nb = C.c_uint64()
        call("hps_nn_conv_tc_tile_bytes", dp, C.byref(nb))
        if nb.value == 0:
            self._tiles[key] = (None, self._wver)
            return None
        t = hit[0] if hit is not None and hit[0] is not None else \
            self.torch.empty(int(nb.value), dtype=self.torch.uint8, device=self.device)
        call("hps_nn_conv_tc_prepare", dp, _p(self.wb[li]), _p(t), None)
        self._tiles[key] = (t, self._wver)
        return t

    def tensor_core_errors(self):
        """1 when a tensor-core layer's bounded pipeline wait gave up since
        the network was made."""
        return int(self._tc_err.item())

    def forward(self, x):
        """x: [B, 2, NZ, NR] BF16.  Returns (ins, acts, outs): layer l reads
        ins[l], acts[l] is its output after ReLU (the backward mask) and
        outs[l] what the next layer reads (after the plane-mean broadcast or
        the skip addition); outs[-1] is the prediction."""
        torch = self.torch
        B = x.shape[0]
        ins, acts, outs = [], [], []
        cur = x
        for li, dims in enumerate(layer_shapes(B, x.shape[2], x.shape[3])):
            _, ci, co, h, w, s, u = dims
            ho, wo = (h * u - 1) // s + 1, (w * u - 1) // s + 1
            y = torch.empty((B, co, ho, wo), dtype=torch.bfloat16, device=self.device)
            tiles = self._layer_tiles(li, dims) if self.tensor_cores and B >= 2 else None
            if tiles is not None:
                call("hps_nn_conv_forward_tiles", dims.ctypes.data_as(C.POINTER(C.c_int)), _p(cur), _p(tiles),
                     _p(self.b[li]), int(ARCH[li][4]), None, _p(y), _p(self._tc_err), None)
            else:
                call("hps_nn_conv_forward", dims.ctypes.data_as(C.POINTER(C.c_int)), _p(cur), _p(self.wb[li]),
                     _p(self.b[li]), int(ARCH[li][4]), None, _p(y), None)
            ins.append(cur)
            acts.append(y)
            out = y
            if li == GMEAN_AFTER:
                out = y.clone()
                call("hps_nn_gmean_forward", _p(out), B * co, ho * wo, None)
            if li in SKIP:
                out = torch.empty_like(y)
                call("hps_nn_add", _p(y), _p(outs[SKIP[li]]), _p(out), y.numel(), 1, None)
            outs.append(out)
            cur = out
        return ins, acts, outs

    def backward(self, fwd, dy):
        """dy: FP32 gradient of the loss with respect to the prediction.
        Returns [dW_l], [db_l]."""
        torch = self.torch
        ins, acts, outs = fwd
        B = ins[0].shape[0]
        dims_all = layer_shapes(B, ins[0].shape[2], ins[0].shape[3])
        n = len(ARCH)
        dws, dbs = [None] * n, [None] * n
        gout = [None] * n  # gradient with respect to outs[l]
        gout[-1] = dy

        def accumulate(l, g):
            if gout[l] is None:
                gout[l] = g
            else:
                s = torch.empty_like(g)
                call("hps_nn_add", _p(gout[l]), _p(g), _p(s), g.numel(), 0, None)
                gout[l] = s

        for li in reversed(range(n)):
            g = gout[li]
            if li in SKIP:
                accumulate(SKIP[li], g)  # outs[li] = acts[li] + outs[skip]
            if li == GMEAN_AFTER:
                g = g.clone()
                call("hps_nn_gmean_backward", _p(g), g.shape[0] * g.shape[1], g.shape[2] * g.shape[3], None)
            dims = dims_all[li]
            x, y = ins[li], acts[li]
            dz = torch.empty(y.shape, dtype=torch.float32, device=self.device)
            dx = torch.empty(x.shape, dtype=torch.float32, device=self.device) if li > 0 else None
            dw = torch.empty_like(self.w[li])
            db = torch.empty_like(self.b[li])
            call("hps_nn_conv_backward", dims.ctypes.data_as(C.POINTER(C.c_int)), _p(x), _p(self.wb[li]), _p(y),
                 int(ARCH[li][4]), _p(g), _p(dz), _p(dx) if dx is not None else None, _p(dw), _p(db), None)
            dws[li], dbs[li] = dw, db
            if dx is not None:
                accumulate(li - 1, dx)
        return dws, dbs

    def loss_grad(self, pred, target, weight=None):
        """Weighted squared error (weight per sample, or none) and its gradient."""
        torch = self.torch
        n = pred.numel()
        nblk = 64
        dpred = torch.empty(pred.shape, dtype=torch.float32, device=self.device)
        part = torch.empty(nblk, dtype=torch.float32, device=self.device)
        call("hps_nn_mse", _p(pred), _p(target), n, _p(weight) if weight is not None else None,
             n // pred.shape[0], _p(dpred), _p(part), nblk, None)
        return float(part.sum().item()) / n, dpred

    def adam(self, dws, dbs, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        self._wver += 1  # the BF16 weights change below
        params = list(zip(self.w, self.wb, dws)) + [(b, None, db) for b, db in zip(self.b, dbs)]
        for k, (p, pb, g) in enumerate(params):
            call("hps_nn_adam", _p(p), _p(pb) if pb is not None else None, _p(g), _p(self.m[k]), _p(self.v[k]),
                 p.numel(), lr, b1, b2, eps, self.step_count, None)

    def train_step(self, x, target, weight=None, lr=1e-3):
        fwd = self.forward(x)
        loss, dpred = self.loss_grad(fwd[2][-1], target, weight)
        dws, dbs = self.backward(fwd, dpred)
        self.adam(dws, dbs, lr)
        return loss

    def predict(self, x):
        """FP32 [B, 2, NZ, NR] normalised prediction."""
        return self.forward(x)[2][-1].float()


def _bf16_bits(a):
    """uint16 BF16 bits of float32 values, rounded to nearest even (as the
    device's float -> bfloat16 conversion)."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def export(state):
    """What a solver takes (SpaceCharge.set_surrogate): the layer table,
    BF16 weight bits and FP32 biases of a saved network state."""
    n = len(ARCH)
    skip = np.full(n, -1, np.int32)
    for l, s in SKIP.items():
        skip[l] = s
    return {"arch": np.array(ARCH, np.int32), "gmean_after": GMEAN_AFTER, "skip": skip,
            "weights": [_bf16_bits(np.asarray(state[f"w{i}"], np.float32)) for i in range(n)],
            "biases": [np.asarray(state[f"b{i}"], np.float32) for i in range(n)],
            "out_scale": float(state["out_scale"]), "nr": NR, "nz": NZ}


# ---- scale-free inputs and targets ------------------------------------------
def green_c1(current, frac, freq, num, mass):
    """The solver's Green's-table scale (UpdateFldTbl1Kernel's c1)."""
    return 5721.67 * current * frac / (freq * 1e6 * num * mass)


def make_input(bins, nr, nz, dr, dz, beta):
    """[2, nz, nr] float32: charge / total * nr*nz, and log of the cell
    aspect dz*gamma/dr."""
    q = np.asarray(bins, np.float64).reshape(nz, nr)
    total = q.sum()
    gamma = 1.0 / math.sqrt(1.0 - beta * beta)
    x = np.empty((2, nz, nr), np.float32)
    x[0] = q / total * (nr * nz) if total > 0 else 0.0
    x[1] = math.log(dz * gamma / dr)
    return x, total


def field_scale(dr, dzg, c1, total):
    """E * this = the network's target (before out_scale).  dr^2 / (c1 sum q)
    makes the field scale-free; the extra aspect factor dzg / dr evens out
    its magnitude across cell shapes (a long cell spreads the same charge
    over a longer bunch)."""
    return dr * dzg / (c1 * total)


def make_target(field, nr, nz, dr, dzg, c1, total):
    f = np.asarray(field, np.float64).reshape(nz + 1, nr + 1, 2)[:nz, :nr]
    return (f * field_scale(dr, dzg, c1, total)).transpose(2, 0, 1).astype(np.float32)


# ---- snapshots of the plain solver along small-FODO tracking -----------------
def snapshots(n_runs=48, num=32768, seed=1, precision="fp64", elems=None):
    """(inputs [S, 2, nz, nr], targets [S, 2, nz, nr]) from plain-SCHEFF kicks
    of small-FODO runs with currents U(5, 25) mA and emittance scales
    U(0.5, 2), one snapshot per element."""
    from . import HPSim, lattices as L
    rng = np.random.default_rng(seed)
    elems = elems or L.small_fodo()
    xs, ys = [], []
    for run in range(n_runs):
        cur = rng.uniform(0.005, 0.025)
        scale = rng.uniform(0.5, 2.0)
        tw = list(L.waterbag_twiss())
        for k in (2, 5, 8):
            tw[k] *= scale
        beam = HPSim.Beam(mass=939.294, charge=-1.0, current=cur, num=num, precision=precision)
        beam.set_waterbag(*tw, 0.0, 0.75, 201.25, int(rng.integers(1, 2 ** 31)))
        beam.set_ref_w(0.75)
        sc = HPSim.SpaceCharge(NR, NZ, 0.1, 0)
        sc.set_remesh_threshold(0.0)
        sim = HPSim.Simulator(beam, HPSim.BeamLine(elements=elems), sc)
        sim.use_graph(False)
        c1 = green_c1(cur, 1.0, 201.25, num, 939.294)
        bins = np.empty(NR * NZ)
        field = np.empty((NZ + 1) * (NR + 1) * 2)
        mesh = np.empty(7)
        for i in range(len(elems)):
            sim.simulate(i, i)
            call("hps_scheff_snapshot", sc.handle, 1 if precision == "fp32" else 0,
                 bins.ctypes.data_as(C.POINTER(C.c_double)), field.ctypes.data_as(C.POINTER(C.c_double)),
                 mesh.ctypes.data_as(C.POINTER(C.c_double)))
            if int(mesh[0]) != NR or int(mesh[1]) != NZ or mesh[6] == 0:
                continue
            x, total = make_input(bins, NR, NZ, mesh[2], mesh[3], mesh[4])
            if total <= 0:
                continue
            dzg = mesh[3] / math.sqrt(1.0 - mesh[4] * mesh[4])
            xs.append(x)
            ys.append(make_target(field, NR, NZ, mesh[2], dzg, c1, total))
    return np.stack(xs), np.stack(ys)


def train(net, xs, ys, epochs=30, batch=32, lr=2e-3, seed=0, log=None):
    """Adam on the squared error of the scaled targets, the learning rate
    halved every quarter of the epochs; returns the loss history (mean per
    epoch)."""
    torch = net.torch
    rng = np.random.default_rng(seed)
    if net.out_scale == 1.0:
        net.out_scale = float(1.0 / (np.std(ys) + 1e-30))
    X = torch.tensor(xs, dtype=torch.bfloat16, device=net.device)
    Y = torch.tensor(ys * net.out_scale, dtype=torch.float32, device=net.device)
    hist = []
    n = len(xs)
    period = max(1, epochs // 4)
    for ep in range(epochs):
        order = rng.permutation(n)
        tot = 0.0
        for k in range(0, n - batch + 1, batch):
            sel = torch.tensor(order[k:k + batch], device=net.device)
            tot += net.train_step(X[sel].contiguous(), Y[sel].contiguous(), None, lr=lr * (0.5 ** (ep // period)))
        hist.append(tot / max(1, n // batch))
        if net.tensor_core_errors():
            raise RuntimeError("surrogate training: a tensor-core layer's pipeline wait timed out")
        if log:
            log(ep, hist[-1])
    return hist


def relative_error(net, xs, ys):
    """Relative L2 error of the predicted field per snapshot."""
    torch = net.torch
    X = torch.tensor(xs, dtype=torch.bfloat16, device=net.device)
    p = net.predict(X).cpu().numpy() / net.out_scale
    num = np.sqrt(((p - ys) ** 2).reshape(len(xs), -1).sum(1))
    den = np.sqrt((ys ** 2).reshape(len(xs), -1).sum(1))
    return num / den


def relative_error_batched(net, xs, ys, chunk=256):
    return np.concatenate([relative_error(net, xs[k:k + chunk], ys[k:k + chunk]) for k in range(0, len(xs), chunk)])


def save_for_inference(net, path, **meta):
    """The weights rounded to BF16 (what a solver evaluates) and the output
    scale, compressed, with provenance numbers in `meta`."""
    st = net.state()
    for i in range(len(ARCH)):
        w = np.ascontiguousarray(st[f"w{i}"], np.float32)
        st[f"w{i}"] = (_bf16_bits(w).astype(np.uint32) << 16).view(np.float32)
    np.savez_compressed(path, **st, **{f"meta_{k}": np.float64(v) for k, v in meta.items()})


def main(argv=None):
    """python -m hpsim_gb300.surrogate --out net.npz [--runs R --num N
    --epochs E --seed S]: snapshots of plain-SCHEFF small-FODO runs, training
    on this GPU, validation on runs of another seed, the network saved for
    SpaceCharge.set_surrogate."""
    import argparse
    import time
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--out", required=True)
    ap.add_argument("--runs", type=int, default=120)
    ap.add_argument("--val-runs", type=int, default=8)
    ap.add_argument("--num", type=int, default=16384)
    ap.add_argument("--epochs", type=int, default=120)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1)
    a = ap.parse_args(argv)
    t0 = time.time()
    xs, ys = snapshots(n_runs=a.runs, num=a.num, seed=a.seed)
    xv, yv = snapshots(n_runs=a.val_runs, num=a.num, seed=a.seed + 1000)
    t1 = time.time()
    print(f"snapshots: {len(xs)} training, {len(xv)} validation ({t1 - t0:.1f} s)", flush=True)
    net = Network(seed=a.seed)

    def log(ep, loss):
        if ep % 10 == 9 or ep == a.epochs - 1:
            e = relative_error_batched(net, xv, yv)
            print(f"epoch {ep + 1}: loss {loss:.3e}, validation field error median {np.median(e):.4f} "
                  f"p90 {np.percentile(e, 90):.4f}", flush=True)

    train(net, xs, ys, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed, log=log)
    t2 = time.time()
    et, ev = relative_error_batched(net, xs, ys), relative_error_batched(net, xv, yv)
    print(f"training {t2 - t1:.1f} s; field error median train {np.median(et):.4f} validation {np.median(ev):.4f} "
          f"(p90 {np.percentile(ev, 90):.4f})", flush=True)
    save_for_inference(net, a.out, train_snapshots=len(xs), val_snapshots=len(xv), epochs=a.epochs,
                       train_median=np.median(et), val_median=np.median(ev), val_p90=np.percentile(ev, 90))


if __name__ == "__main__":
    main()
