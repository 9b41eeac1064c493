"""Device kernels of the learned centroid correction against the CPU oracle:
symmetry functions, the tensor-core forward pass and (training) the weight
gradients."""
import numpy as np
import pytest

from oracle import surrogate_oracle as so

pytestmark = pytest.mark.gpu


def _torch():
    return pytest.importorskip("torch")


def test_descriptors_match_oracle(gpu_lib):
    torch = _torch()
    q = gpu_lib
    sts = [q.seeded_start(64, 1, 298.0, seed=s) for s in (4, 5)]
    box = sts[0].box_bohr
    pos = torch.tensor(np.stack([st.q for st in sts]), dtype=torch.float64, device="cuda")
    desc = torch.zeros((2, 192, 32), dtype=torch.float32, device="cuda")
    q.sym_descriptors(pos.data_ptr(), 2, 64, box, desc.data_ptr())
    assert q.surrogate_status() == 0
    got = desc.cpu().numpy()
    for c, st in enumerate(sts):
        ref = so.sym_descriptors(st.q, box)
        err = np.abs(got[c] - ref) / (np.abs(ref) + 1e-3)
        assert err.max() < 2e-4, (c, err.max(), np.unravel_index(err.argmax(), err.shape))


def _weights(torch, p):
    dev = {}
    for k in ("w1", "w2", "w3"):
        dev[k] = torch.tensor(p[k], dtype=torch.float32, device="cuda").to(torch.bfloat16).contiguous()
    for k in ("b1", "b2", "b3"):
        dev[k] = torch.tensor(p[k], dtype=torch.float32, device="cuda").contiguous()
    return dev


def test_forward_matches_oracle(gpu_lib):
    torch = _torch()
    q = gpu_lib
    rng = np.random.default_rng(7)
    p = so.init_params(11)
    for k in ("b1", "b2", "b3"):
        p[k] = rng.standard_normal(p[k].shape) * 0.2
    p["b3"][9:] = 0.0
    m = 300  # two full tiles and a partial one
    x = rng.standard_normal((m, 96))
    dev = _weights(torch, p)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda").to(torch.bfloat16).contiguous()
    yd = torch.full((m, 16), np.nan, dtype=torch.float32, device="cuda")
    w = q.MlpWeights(*[dev[k].data_ptr() for k in ("w1", "w2", "w3", "b1", "b2", "b3")])
    q.mlp_forward(w, xd.data_ptr(), m, yd.data_ptr())
    assert q.surrogate_status() == 0
    y = yd.cpu().numpy().astype(np.float64)
    ref, _ = so.mlp_forward(p, x)
    scale = np.abs(ref).max()
    assert np.all(np.isfinite(y))
    assert np.abs(y - ref).max() < 2e-2 * scale, np.abs(y - ref).max() / scale
    assert np.sqrt(np.mean((y - ref) ** 2)) < 3e-3 * scale


def _flat(p):
    return np.concatenate([p[k].reshape(-1) for k in ("w1", "w2", "w3", "b1", "b2", "b3")])


class _Dev:
    """Device buffers of one parameter vector (FP32 masters, BF16 weight copies)."""

    def __init__(self, torch, q, p):
        self.torch, self.q = torch, q
        self.params = torch.tensor(_flat(p), dtype=torch.float32, device="cuda")
        self.wbf = self.params[: q.MLP_NW].to(torch.bfloat16).contiguous()
        self.m1 = torch.zeros_like(self.params)
        self.m2 = torch.zeros_like(self.params)

    def weights(self):
        q, P, B = self.q, self.params.data_ptr(), self.wbf.data_ptr()
        return q.MlpWeights(B, B + 2 * 64 * 96, B + 2 * (64 * 96 + 64 * 64), P + 4 * q.MLP_NW,
                            P + 4 * (q.MLP_NW + 64), P + 4 * (q.MLP_NW + 128))


def _train_batch(torch, q, dev, x, t, max_ctas):
    m = x.shape[0]
    xd = torch.tensor(x, dtype=torch.float32, device="cuda").to(torch.bfloat16).contiguous()
    td = torch.tensor(t, dtype=torch.float32, device="cuda").contiguous()
    part = torch.zeros((max_ctas, q.MLP_NPARAMS + 1), dtype=torch.float32, device="cuda")
    grad = torch.zeros(q.MLP_NPARAMS + 1, dtype=torch.float32, device="cuda")
    q.mlp_train_batch(dev.weights(), xd.data_ptr(), td.data_ptr(), m, 2.0 / (m * 9), part.data_ptr(), max_ctas,
                      grad.data_ptr())
    assert q.surrogate_status() == 0
    return grad.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("max_ctas", [1, 64])
def test_train_gradients_match_oracle(gpu_lib, max_ctas):
    torch = _torch()
    q = gpu_lib
    rng = np.random.default_rng(9)
    p = so.init_params(13)
    for k in ("b1", "b2", "b3"):
        p[k] = rng.standard_normal(p[k].shape) * 0.1
    p["b3"][9:] = 0.0
    m = 300
    x = rng.standard_normal((m, 96))
    t = np.zeros((m, 16))
    t[:, :9] = rng.standard_normal((m, 9))
    dev = _Dev(torch, q, p)
    got = _train_batch(torch, q, dev, x, t, max_ctas)
    y, cache = so.mlp_forward(p, x)
    loss, dy = so.mse_loss(y, t)
    ref = so.mlp_backward(cache, dy)
    assert abs(got[-1] / (m * 9) - loss) < 1e-3 * loss
    off = 0
    for k in ("w1", "w2", "w3", "b1", "b2", "b3"):
        n = p[k].size
        g, r = got[off:off + n], ref[k].reshape(-1)
        rel = np.linalg.norm(g - r) / np.linalg.norm(r)
        assert rel < 2e-2, (k, rel)
        off += n


def test_adam_training_reduces_the_loss(gpu_lib):
    """Fit the outputs of a fixed teacher network: the device trainer (tensor-core
    forward/backward, fixed-order gradient sum, Adam) must cut the loss severalfold."""
    torch = _torch()
    q = gpu_lib
    rng = np.random.default_rng(21)
    teacher = so.init_params(5)
    m = 2048
    x = rng.standard_normal((m, 96))
    t, _ = so.mlp_forward(teacher, x)
    t[:, 9:] = 0.0
    dev = _Dev(torch, q, so.init_params(6))
    xd = torch.tensor(x, dtype=torch.float32, device="cuda").to(torch.bfloat16).contiguous()
    td = torch.tensor(t, dtype=torch.float32, device="cuda").contiguous()
    part = torch.zeros((256, q.MLP_NPARAMS + 1), dtype=torch.float32, device="cuda")
    grad = torch.zeros(q.MLP_NPARAMS + 1, dtype=torch.float32, device="cuda")
    losses = []
    for step in range(1, 301):
        q.mlp_train_batch(dev.weights(), xd.data_ptr(), td.data_ptr(), m, 2.0 / (m * 9), part.data_ptr(), 256,
                          grad.data_ptr())
        if step in (1, 300):
            losses.append(float(grad[-1].item()) / (m * 9))
        q.adam_step(dev.params.data_ptr(), dev.m1.data_ptr(), dev.m2.data_ptr(), grad.data_ptr(), q.MLP_NPARAMS, step,
                    3e-3, dev.wbf.data_ptr(), q.MLP_NW)
    assert q.surrogate_status() == 0
    assert losses[1] < 0.2 * losses[0], losses
