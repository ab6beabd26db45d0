"""The learned constitutive surrogate for material 7 (anisotropic GOH + Prony).

``Surrogate`` wraps the ftgpu_surrogate_* entry points: generate training
samples from the plain law on the GPU, train the BF16 MLP with the GPU's
forward / backward / Adam kernels, predict.  The network predicts
S_iso = S_lin(E, a0) + s0 * out_scale * |E|^2 * NN(x); ``linear_part``,
``features`` and ``e2_of`` are the host mirror of ``surrogate_features`` in
csrc/ft_mlp.cuh, and ``predict`` runs that reconstruction on the device.

The default sampling box (principal stretches 0.77..1.19) covers the default
trust region |E|_F^2 <= 0.04 (every |E_ii| <= 0.2), where the network is used.
"""
import ctypes as C

import numpy as np

from . import _check, lib

N_IN, N_HID, N_OUT = 16, 128, 8
USED_IN, USED_OUT = 9, 6
STRAIN_SCALE = 0.5
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
    return L


def linear_part(E, a0, mu, k1, kappa):
    """S_lin (Voigt 11,22,33,23,13,12) for strains E[n,6] (tensor shear) and fibres a0[n,3]."""
    E = np.asarray(E, np.float64)
    a0 = np.asarray(a0, np.float64)
    tr3 = (E[:, 0] + E[:, 1] + E[:, 2]) / 3.0
    aEa = (a0[:, 0] ** 2 * E[:, 0] + a0[:, 1] ** 2 * E[:, 1] + a0[:, 2] ** 2 * E[:, 2]
           + 2 * (a0[:, 1] * a0[:, 2] * E[:, 3] + a0[:, 0] * a0[:, 2] * E[:, 4]
                  + a0[:, 0] * a0[:, 1] * E[:, 5]))
    c4 = 1.0 - 3.0 * kappa
    Ea = 2.0 * c4 * (aEa - tr3)
    f = np.where(Ea > 0, 2.0 * k1 * c4 * Ea, 0.0)
    S = np.empty_like(E)
    S[:, 0] = 2 * mu * (E[:, 0] - tr3) + f * (a0[:, 0] ** 2 - 1 / 3)
    S[:, 1] = 2 * mu * (E[:, 1] - tr3) + f * (a0[:, 1] ** 2 - 1 / 3)
    S[:, 2] = 2 * mu * (E[:, 2] - tr3) + f * (a0[:, 2] ** 2 - 1 / 3)
    S[:, 3] = 2 * mu * E[:, 3] + f * a0[:, 1] * a0[:, 2]
    S[:, 4] = 2 * mu * E[:, 4] + f * a0[:, 0] * a0[:, 2]
    S[:, 5] = 2 * mu * E[:, 5] + f * a0[:, 0] * a0[:, 1]
    return S


def features(E, a0):
    x = np.zeros((len(E), N_IN), np.float32)
    x[:, :6] = np.asarray(E) / STRAIN_SCALE
    x[:, 6:9] = a0
    return x


def e2_of(E):
    E = np.asarray(E)
    e2 = E[:, 0] ** 2 + E[:, 1] ** 2 + E[:, 2] ** 2 + 2 * (E[:, 3] ** 2 + E[:, 4] ** 2 + E[:, 5] ** 2)
    return np.maximum(e2, E2_FLOOR)


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
