"""FP64 restatement of the surrogate MLP (test infrastructure: the checker of
the GPU's BF16 tensor-core forward / backward kernels).

Same network as femtech_gb300/csrc/ft_mlp.cu: 16 -> 128 -> 128 -> 128 -> 8,
SiLU, parameter vector layout W0[128][16] b0 W1[128][128] b1 W2[128][128] b2
W3[8][128] b3; loss = mean over (rows, 6 used outputs) of the squared error.
``quantize=True`` rounds inputs, weights and hidden activations to BF16 the
way the GPU stores them, so the comparison isolates accumulation error.  The
GPU evaluates the activation on BF16 pairs, SiLU(z) = h + h tanh(h) with
h = z / 2 rounded to BF16, tanh rounded to BF16 and the fused multiply-add
rounded once; ``quantize=True`` follows those roundings (with an exact tanh,
so hardware tanh approximation remains a small difference).  The backward
pass uses the exact SiLU derivative of the FP32 pre-activation, as the GPU.
"""
import numpy as np

NI, NH, NO, NU = 16, 128, 8, 6
OFF = {}
_o = 0
for _name, _n in (("W0", NH * NI), ("b0", NH), ("W1", NH * NH), ("b1", NH), ("W2", NH * NH),
                  ("b2", NH), ("W3", NO * NH), ("b3", NO)):
    OFF[_name] = (_o, _o + _n)
    _o += _n
NPARAMS = _o


def bf16(a):
    """Round to bfloat16 (nearest even) and back to float64."""
    a32 = np.asarray(a, np.float32)
    b = a32.view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    g = {k: np.asarray(p[a:b], np.float64) for k, (a, b) in OFF.items()}
    g["W0"] = g["W0"].reshape(NH, NI)
    g["W1"] = g["W1"].reshape(NH, NH)
    g["W2"] = g["W2"].reshape(NH, NH)
    g["W3"] = g["W3"].reshape(NO, NH)
    return g


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def silu_bf16(z):
    """The GPU's activation: h = bf16(z / 2), bf16(h + h * bf16(tanh(h)))."""
    h = bf16(0.5 * np.asarray(z, np.float64))
    return bf16(h + h * bf16(np.tanh(h)))


def forward(p, x, quantize=True):
    q = bf16 if quantize else (lambda a: np.asarray(a, np.float64))
    act = silu_bf16 if quantize else silu
    w = unpack(p)
    x = q(x)
    z1 = x @ q(w["W0"]).T + w["b0"]
    h1 = act(z1)
    z2 = h1 @ q(w["W1"]).T + w["b1"]
    h2 = act(z2)
    z3 = h2 @ q(w["W2"]).T + w["b2"]
    h3 = act(z3)
    y = h3 @ q(w["W3"]).T + w["b3"]
    return y, (x, z1, h1, z2, h2, z3, h3)


def loss_and_grad(p, x, t, quantize=True):
    q = bf16 if quantize else (lambda a: np.asarray(a, np.float64))
    w = unpack(p)
    y, (x, z1, h1, z2, h2, z3, h3) = forward(p, x, quantize)
    m = len(x)
    d = np.zeros_like(y)
    d[:, :NU] = y[:, :NU] - np.asarray(t, np.float64)[:, :NU]
    loss = float(np.sum(d * d) / (m * NU))
    dy = q(2.0 * d / (m * NU))
    g = {}
    g["W3"] = dy.T @ h3
    g["b3"] = dy.sum(0)
    dz3 = q((dy @ q(w["W3"])) * dsilu(z3))
    g["W2"] = dz3.T @ h2
    g["b2"] = dz3.sum(0)
    dz2 = q((dz3 @ q(w["W2"])) * dsilu(z2))
    g["W1"] = dz2.T @ h1
    g["b1"] = dz2.sum(0)
    dz1 = q((dz2 @ q(w["W1"])) * dsilu(z1))
    g["W0"] = dz1.T @ x
    g["b0"] = dz1.sum(0)
    out = np.zeros(NPARAMS)
    for k, (a, b) in OFF.items():
        out[a:b] = g[k].ravel()
    return loss, out
