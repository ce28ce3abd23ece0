"""The surrogate's host-side helpers without a GPU: BF16 rounding of the
exported weights against torch's float -> bfloat16 conversion, the export
layout a solver takes, and the inference save format."""
import numpy as np
import pytest

from hpsim_gb300 import surrogate as S

torch = pytest.importorskip("torch")


def test_bf16_bits_round_like_torch():
    rng = np.random.default_rng(0)
    v = np.concatenate([rng.normal(size=4096).astype(np.float32) * 10.0 ** rng.integers(-8, 8, 4096),
                        np.array([0.0, -0.0, 1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 3.0e38, -2.5e-39], np.float32)])
    ref = torch.tensor(v).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(S._bf16_bits(v), ref)


def _state(seed=0):
    rng = np.random.default_rng(seed)
    st = {f"w{i}": rng.normal(size=(co, ci, 3, 3)).astype(np.float32) for i, (ci, co, *_) in enumerate(S.ARCH)}
    st.update({f"b{i}": rng.normal(size=co).astype(np.float32) for i, (_, co, *_) in enumerate(S.ARCH)})
    st["out_scale"] = np.float64(3.5)
    return st


def test_export_layout():
    st = _state()
    ex = S.export(st)
    assert ex["arch"].shape == (len(S.ARCH), 5) and ex["arch"].dtype == np.int32
    assert ex["nr"] == S.NR and ex["nz"] == S.NZ and ex["out_scale"] == 3.5
    assert ex["gmean_after"] == S.GMEAN_AFTER
    assert [int(k) for k in ex["skip"]] == [S.SKIP.get(i, -1) for i in range(len(S.ARCH))]
    for i, (ci, co, *_) in enumerate(S.ARCH):
        assert ex["weights"][i].dtype == np.uint16 and ex["weights"][i].shape == (co, ci, 3, 3)
        assert np.array_equal(ex["biases"][i], st[f"b{i}"])
    # layer shapes chain to the mesh (what the solver checks before attaching)
    c, h, w = 2, S.NZ, S.NR
    for ci, co, s, u, _ in S.ARCH:
        assert ci == c
        h, w, c = (h * u - 1) // s + 1, (w * u - 1) // s + 1, co
    assert (c, h, w) == (2, S.NZ, S.NR)


def test_saved_network_holds_bf16_weights(tmp_path):
    class Net:
        def state(self):
            return _state(1)

    path = tmp_path / "net.npz"
    S.save_for_inference(Net(), path, val_median=0.02)
    z = np.load(path)
    assert float(z["meta_val_median"]) == 0.02
    for i in range(len(S.ARCH)):
        w = z[f"w{i}"]
        assert not np.any(w.view(np.uint32) & 0xFFFF)  # exactly representable in BF16
        assert np.array_equal(S._bf16_bits(w), S._bf16_bits(_state(1)[f"w{i}"]))
