"""Planar layer system and its response, vectorised over in-plane wavenumbers.

Mirrors smuthi/layers.py: the ``LayerSystem`` geometry (:17-203), Fresnel
coefficients and transfer / scattering matrices (:206-333) and the layer
system response matrix (:336-380). Where the reference loops over kappa in
Python (and memoises per kappa), the 2 x 2 algebra here runs on arrays of
shape (2, 2, K).
"""
import numpy as np

from . import fields as flds


class LayerSystem:
    """Stack of planar layers; first and last are half-spaces (thickness 0)."""

    def __init__(self, thicknesses=None, refractive_indices=None):
        if thicknesses is None:
            thicknesses = [0, 0]
        if refractive_indices is None:
            refractive_indices = [1, 1]
        if len(thicknesses) != len(refractive_indices):
            raise ValueError('%d layer thicknesses but %d refractive indices'
                             % (len(thicknesses), len(refractive_indices)))
        self.thicknesses = list(thicknesses)
        self.thicknesses[0] = 0
        self.thicknesses[-1] = 0
        self.refractive_indices = list(refractive_indices)

    def is_degenerate(self):
        """True for two half-spaces of the same material (no layer-mediated coupling)."""
        return self.thicknesses == [0, 0] and self.refractive_indices[0] == self.refractive_indices[-1]

    def number_of_layers(self):
        return len(self.thicknesses)

    def lower_zlimit(self, i):
        return -np.inf if i == 0 else sum(self.thicknesses[1:i])

    def upper_zlimit(self, i):
        return np.inf if i == self.number_of_layers() - 1 else sum(self.thicknesses[1:i + 1])

    def reference_z(self, i):
        return self.upper_zlimit(i) if i == 0 else self.lower_zlimit(i)

    def layer_number(self, z):
        """Layer containing height z (a point on an interface belongs to the upper layer)."""
        top = 0
        num = 0
        for d in self.thicknesses[1:]:
            if z < top:
                break
            num += 1
            top += d
        return num

    def wavenumber(self, layer_number, vacuum_wavelength):
        return self.refractive_indices[layer_number] * flds.angular_frequency(vacuum_wavelength)


# ---------------------------------------------------------------- 2x2 algebra on (2, 2, K) arrays
def _mm(a, b):
    return np.einsum('ijk,jlk->ilk', a, b)


def _inv(a):
    det = a[0, 0] * a[1, 1] - a[0, 1] * a[1, 0]
    return np.array([[a[1, 1], -a[0, 1]], [-a[1, 0], a[0, 0]]]) / det


def _eye(K):
    e = np.zeros((2, 2, K), complex)
    e[0, 0] = e[1, 1] = 1
    return e


def _kz(n, kpar, omega):
    kz = np.sqrt((omega * n) ** 2 - kpar ** 2 + 0j)
    return np.where(kz.imag < 0, -kz, kz)


def _interface(pol, kz1, kz2, n1, n2):
    if pol == 0:
        r = (kz1 - kz2) / (kz1 + kz2)
        t = 2 * kz1 / (kz1 + kz2)
    else:
        r = (n2 ** 2 * kz1 - n1 ** 2 * kz2) / (n2 ** 2 * kz1 + n1 ** 2 * kz2)
        t = 2 * n1 * n2 * kz1 / (n2 ** 2 * kz1 + n1 ** 2 * kz2)
    one = np.ones_like(r)
    return np.array([[one, r], [r, one]]) / t


def _propagation(kz, d):
    z = np.zeros_like(kz)
    return np.array([[np.exp(-1j * kz * d), z], [z, np.exp(1j * kz * d)]])


def transfer_matrix(pol, layer_d, layer_n, kpar, omega):
    kpar = np.atleast_1d(kpar)
    kzs = [_kz(n, kpar, omega) for n in layer_n]
    t = _eye(len(kpar))
    for i in range(len(layer_d) - 1):
        t = _mm(t, _mm(_propagation(kzs[i], layer_d[i]), _interface(pol, kzs[i], kzs[i + 1], layer_n[i],
                                                                      layer_n[i + 1])))
    return t


def scattering_matrix(pol, layer_d, layer_n, kpar, omega):
    kpar = np.atleast_1d(kpar)
    kzs = [_kz(n, kpar, omega) for n in layer_n]
    s = _eye(len(kpar))
    for i in range(len(layer_d) - 1):
        t = _mm(_propagation(kzs[i], layer_d[i]), _interface(pol, kzs[i], kzs[i + 1], layer_n[i], layer_n[i + 1]))
        den = t[0, 0] - s[0, 1] * t[1, 0]
        s00 = s[0, 0] / den
        s01 = (s[0, 1] * t[1, 1] - t[0, 1]) / den
        s10 = s[1, 1] * t[1, 0] * s00 + s[1, 0]
        s11 = s[1, 1] * t[1, 0] * s01 + s[1, 1] * t[1, 1]
        s = np.array([[s00, s01], [s10, s11]])
    return s


def layersystem_response_matrix(pol, layer_d, layer_n, kpar, omega, fromlayer, tolayer):
    """Response matrix L (2, 2, K): amplitudes in ``tolayer`` excited from ``fromlayer``."""
    layer_d = list(layer_d)
    layer_n = list(layer_n)
    kpar = np.atleast_1d(np.asarray(kpar))
    K = len(kpar)
    zero = np.zeros(K, complex)
    if fromlayer == 0:
        s = scattering_matrix(pol, layer_d, layer_n, kpar, omega)
        lmat = np.array([[zero, zero], [s[1, 0], zero]])
    elif fromlayer == len(layer_d) - 1:
        s = scattering_matrix(pol, layer_d, layer_n, kpar, omega)
        lmat = np.array([[zero, s[0, 1]], [zero, zero]])
    else:
        sa = scattering_matrix(pol, [0] + layer_d[fromlayer:], [layer_n[fromlayer]] + layer_n[fromlayer:], kpar,
                               omega)
        sb = scattering_matrix(pol, layer_d[:fromlayer] + [0], layer_n[:fromlayer] + [layer_n[fromlayer]], kpar,
                               omega)
        one = np.ones(K, complex)
        lmat = _mm(_inv(np.array([[one, -sb[0, 1]], [-sa[1, 0], one]])),
                   np.array([[zero, sb[0, 1]], [sa[1, 0], zero]]))
    if tolayer > fromlayer:
        tm = transfer_matrix(pol, layer_d[fromlayer:tolayer + 1], layer_n[fromlayer:tolayer + 1], kpar, omega)
        add = np.zeros((2, 2, K), complex)
        add[0, 0] = 1
        lmat = _mm(_inv(tm), lmat + add)
    elif tolayer < fromlayer:
        tm = transfer_matrix(pol, layer_d[tolayer:fromlayer + 1], layer_n[tolayer:fromlayer + 1], kpar, omega)
        add = np.zeros((2, 2, K), complex)
        add[1, 1] = 1
        lmat = _mm(tm, lmat + add)
    return np.asarray(lmat, dtype=complex)
