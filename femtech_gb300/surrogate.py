"""The learned constitutive surrogate for material 7 (anisotropic GOH + Prony).

``Surrogate`` wraps the ftgpu_surrogate_* entry points: generate training
samples from the plain law on the GPU, train the BF16 MLP with the GPU's
forward / backward / Adam kernels, predict.  The network predicts
S_iso = S_lin(E, a0) + s0 * out_scale * |E|^2 * NN(x); ``linear_part``,
``features`` and ``e2_of`` are the host mirror of ``surrogate_features`` in
csrc/ft_mlp.cuh (S_lin uses the exact fibre strain Ebar for the fibre switch),
and ``predict`` runs that reconstruction on the device.

The default sampling box (principal stretches 0.77..1.19) covers the default
trust region |E|_F^2 <= 0.04 (every |E_ii| <= 0.2), where the network is used.
"""
import ctypes as C

import numpy as np

from . import _check, lib

N_IN, N_HID, N_OUT = 16, 128, 8
USED_IN, USED_OUT = 11, 6
STRAIN_SCALE = 0.2
E2_FLOOR = 1e-14
TRUST_E2 = 0.04
STRETCH_LO, STRETCH_HI = 0.77, 1.19


def _bind():
    L = lib()
    vp = C.c_void_p
    L.ftgpu_surrogate_create.argtypes = [C.POINTER(vp), C.c_int, vp, C.c_ulonglong]
    L.ftgpu_surrogate_destroy.argtypes = [vp]
    L.ftgpu_surrogate_generate.argtypes = [vp, C.c_longlong, C.c_ulonglong, C.c_double, C.c_double]
    L.ftgpu_surrogate_train.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.POINTER(C.c_double)]
    L.ftgpu_surrogate_forward.argtypes = [vp, C.c_longlong, vp, vp]
    L.ftgpu_surrogate_gradient.argtypes = [vp, C.c_longlong, vp, vp, vp, C.POINTER(C.c_double)]
    L.ftgpu_surrogate_params.argtypes = [vp, vp, vp]
    L.ftgpu_surrogate_samples.argtypes = [vp, C.c_longlong, vp, vp]
    L.ftgpu_surrogate_num_params.restype = C.c_int
    L.ftgpu_surrogate_predict.argtypes = [vp, C.c_longlong, vp, vp, vp]
    L.ftgpu_surrogate_output_scale.argtypes = [vp, C.POINTER(C.c_double)]
    L.ftgpu_surrogate_gemm_path.argtypes = [vp, C.c_int]
    return L


def fibre_strain(E, a0, kappa):
    """Exact GOH fibre strain kappa (I1bar - 3) + (1 - 3 kappa)(I4bar - 1)."""
    X = 2.0 * np.asarray(E, np.float64)
    a0 = np.asarray(a0, np.float64)
    tr = X[:, 0] + X[:, 1] + X[:, 2]
    i2 = ((X[:, 0] * X[:, 1] - X[:, 5] ** 2) + (X[:, 0] * X[:, 2] - X[:, 4] ** 2)
          + (X[:, 1] * X[:, 2] - X[:, 3] ** 2))
    i3 = (X[:, 0] * (X[:, 1] * X[:, 2] - X[:, 3] ** 2) - X[:, 5] * (X[:, 5] * X[:, 2] - X[:, 3] * X[:, 4])
          + X[:, 4] * (X[:, 5] * X[:, 3] - X[:, 1] * X[:, 4]))
    jm = np.expm1(-np.log1p(tr + i2 + i3) / 3.0)
    aXa = (a0[:, 0] ** 2 * X[:, 0] + a0[:, 1] ** 2 * X[:, 1] + a0[:, 2] ** 2 * X[:, 2]
           + 2 * (a0[:, 1] * a0[:, 2] * X[:, 3] + a0[:, 0] * a0[:, 2] * X[:, 4]
                  + a0[:, 0] * a0[:, 1] * X[:, 5]))
    return kappa * (jm * (3.0 + tr) + tr) + (1.0 - 3.0 * kappa) * (jm * (1.0 + aXa) + aXa)


def linear_part(E, a0, mu, k1, kappa):
    """S_lin (Voigt 11,22,33,23,13,12) for strains E[n,6] (tensor shear) and fibres a0[n,3]:
    2 mu dev E + 2 k1 (1 - 3 kappa) max(Ebar, 0) dev(a0 a0), Ebar the exact fibre strain."""
    E = np.asarray(E, np.float64)
    a0 = np.asarray(a0, np.float64)
    tr3 = (E[:, 0] + E[:, 1] + E[:, 2]) / 3.0
    c4 = 1.0 - 3.0 * kappa
    Eb = fibre_strain(E, a0, kappa)
    f = np.where(Eb > 0, 2.0 * k1 * c4 * Eb, 0.0)
    S = np.empty_like(E)
    S[:, 0] = 2 * mu * (E[:, 0] - tr3) + f * (a0[:, 0] ** 2 - 1 / 3)
    S[:, 1] = 2 * mu * (E[:, 1] - tr3) + f * (a0[:, 1] ** 2 - 1 / 3)
    S[:, 2] = 2 * mu * (E[:, 2] - tr3) + f * (a0[:, 2] ** 2 - 1 / 3)
    S[:, 3] = 2 * mu * E[:, 3] + f * a0[:, 1] * a0[:, 2]
    S[:, 4] = 2 * mu * E[:, 4] + f * a0[:, 0] * a0[:, 2]
    S[:, 5] = 2 * mu * E[:, 5] + f * a0[:, 0] * a0[:, 1]
    return S


def e2_of(E):
    E = np.asarray(E)
    e2 = E[:, 0] ** 2 + E[:, 1] ** 2 + E[:, 2] ** 2 + 2 * (E[:, 3] ** 2 + E[:, 4] ** 2 + E[:, 5] ** 2)
    return np.maximum(e2, E2_FLOOR)


def features(E, a0, kappa):
    """Network inputs: E / |E|_F, |E|_F / 0.2, a0, Ebar / |E|_F."""
    E = np.asarray(E, np.float64)
    en = np.sqrt(e2_of(E))
    x = np.zeros((len(E), N_IN), np.float32)
    x[:, :6] = E / en[:, None]
    x[:, 6] = en / STRAIN_SCALE
    x[:, 7:10] = a0
    x[:, 10] = fibre_strain(E, a0, kappa) / en
    return x


def strain_of(x):
    """Green strain back from (BF16-rounded) features."""
    x = np.asarray(x, np.float64)
    return x[:, :6] * (x[:, 6] * STRAIN_SCALE)[:, None]


class Surrogate:
    def __init__(self, props, device=0, seed=0):
        self.L = _bind()
        self.props = np.zeros(9)
        self.props[: len(props)] = props
        self.mu, self.k1, self.kappa = self.props[1], self.props[3], self.props[7]
        self.s0 = self.mu + self.k1
        self.h = C.c_void_p()
        _check(self.L.ftgpu_surrogate_create(C.byref(self.h), int(device), self.props.ctypes.data,
                                             int(seed)))
        self.nparams = self.L.ftgpu_surrogate_num_params()

    def close(self):
        if getattr(self, "h", None):
            self.L.ftgpu_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def generate(self, n, seed=1, lo=STRETCH_LO, hi=STRETCH_HI):
        _check(self.L.ftgpu_surrogate_generate(self.h, int(n), int(seed), float(lo), float(hi)))

    def train(self, epochs=2, batch=8192, lr=2e-3):
        loss = C.c_double()
        _check(self.L.ftgpu_surrogate_train(self.h, int(epochs), int(batch), float(lr), C.byref(loss)))
        return loss.value

    def gemm_path(self, tensor_cores=True):
        """Training GEMMs on tcgen05 with TMEM accumulators (True, the
        default) or on the warp-level mma.sync kernel (False, a cross-check)."""
        _check(self.L.ftgpu_surrogate_gemm_path(self.h, 1 if tensor_cores else 0))

    def forward(self, x):
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((len(x), N_OUT), np.float32)
        _check(self.L.ftgpu_surrogate_forward(self.h, len(x), x.ctypes.data, y.ctypes.data))
        return y

    def gradient(self, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        g = np.zeros(self.nparams, np.float32)
        loss = C.c_double()
        _check(self.L.ftgpu_surrogate_gradient(self.h, len(x), x.ctypes.data, t.ctypes.data,
                                               g.ctypes.data, C.byref(loss)))
        return g, loss.value

    @property
    def params(self):
        p = np.zeros(self.nparams, np.float32)
        _check(self.L.ftgpu_surrogate_params(self.h, p.ctypes.data, None))
        return p

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        _check(self.L.ftgpu_surrogate_params(self.h, None, p.ctypes.data))

    @property
    def out_scale(self):
        """RMS of the generated targets: the network output is in these units."""
        v = C.c_double()
        _check(self.L.ftgpu_surrogate_output_scale(self.h, C.byref(v)))
        return v.value

    def samples(self, n):
        x = np.zeros((n, N_IN), np.float32)
        t = np.zeros((n, N_OUT), np.float32)
        _check(self.L.ftgpu_surrogate_samples(self.h, int(n), x.ctypes.data, t.ctypes.data))
        return x, t

    def predict(self, E, a0):
        """S_iso (Voigt) from Green strains E[n,6] and fibres a0[n,3], on the device."""
        E = np.ascontiguousarray(E, np.float64)
        a0 = np.ascontiguousarray(a0, np.float64)
        S = np.zeros((len(E), 6))
        _check(self.L.ftgpu_surrogate_predict(self.h, len(E), E.ctypes.data, a0.ctypes.data,
                                              S.ctypes.data))
        return S
