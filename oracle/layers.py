"""Oracle: planar layer system (smuthi/layers.py). Test infrastructure only."""
import numpy as np


class LayerSystem:
    """smuthi/layers.py:17-203 -- geometry part of ``LayerSystem``."""

    def __init__(self, thicknesses=(0, 0), refractive_indices=(1, 1)):
        self.thicknesses = list(thicknesses)
        self.thicknesses[0] = 0
        self.thicknesses[-1] = 0
        self.refractive_indices = list(refractive_indices)

    def is_degenerate(self):
        """smuthi/layers.py:44-55."""
        return self.thicknesses == [0, 0] and self.refractive_indices[0] == self.refractive_indices[-1]

    def number_of_layers(self):
        return len(self.thicknesses)

    def lower_zlimit(self, i):
        """smuthi/layers.py:66-83."""
        if i == 0:
            return -np.inf
        return sum(self.thicknesses[1:i])

    def upper_zlimit(self, i):
        """smuthi/layers.py:85-101."""
        if i == self.number_of_layers() - 1:
            return np.inf
        return sum(self.thicknesses[1:i + 1])

    def reference_z(self, i):
        """smuthi/layers.py:103-117."""
        return self.upper_zlimit(i) if i == 0 else self.lower_zlimit(i)

    def layer_number(self, z):
        """smuthi/layers.py:119-139 (interfaces belong to the upper layer)."""
        d = 0
        laynum = 0
        for th in self.thicknesses[1:]:
            if z >= d:
                laynum += 1
                d += th
            else:
                break
        return laynum

    def wavenumber(self, i, vacuum_wavelength):
        return self.refractive_indices[i] * 2 * np.pi / vacuum_wavelength


def _kz(n, kpar, omega):
    kz = np.sqrt((omega * n) ** 2 - kpar ** 2 + 0j)
    return -kz if kz.imag < 0 else kz


def _interface_matrix(pol, kz1, kz2, n1, n2):
    """smuthi/layers.py:206-261 -- (1/t) [[1, r], [r, 1]] with Fresnel r, t."""
    if pol == 0:
        r = (kz1 - kz2) / (kz1 + kz2)
        t = 2 * kz1 / (kz1 + kz2)
    else:
        r = (n2 ** 2 * kz1 - n1 ** 2 * kz2) / (n2 ** 2 * kz1 + n1 ** 2 * kz2)
        t = 2 * n1 * n2 * kz1 / (n2 ** 2 * kz1 + n1 ** 2 * kz2)
    return 1 / t * np.array([[1, r], [r, 1]])


def _propagation_matrix(kz, d):
    """smuthi/layers.py:264-275."""
    return np.array([[np.exp(-1j * kz * d), 0], [0, np.exp(1j * kz * d)]])


def transfer_matrix(pol, layer_d, layer_n, kpar, omega):
    """smuthi/layers.py:278-302."""
    kzs = [_kz(n, kpar, omega) for n in layer_n]
    tmat = np.eye(2)
    for i in range(len(layer_d) - 1):
        dmat = _interface_matrix(pol, kzs[i], kzs[i + 1], layer_n[i], layer_n[i + 1])
        tmat = np.dot(tmat, np.dot(_propagation_matrix(kzs[i], layer_d[i]), dmat))
    return tmat


def scattering_matrix(pol, layer_d, layer_n, kpar, omega):
    """smuthi/layers.py:305-333 -- recursive S-matrix over interfaces."""
    kzs = [_kz(n, kpar, omega) for n in layer_n]
    s = np.eye(2)
    for i in range(len(layer_d) - 1):
        t = np.dot(_propagation_matrix(kzs[i], layer_d[i]),
                   _interface_matrix(pol, kzs[i], kzs[i + 1], layer_n[i], layer_n[i + 1]))
        den = t[0, 0] - s[0, 1] * t[1, 0]
        s00 = s[0, 0] / den
        s01 = (s[0, 1] * t[1, 1] - t[0, 1]) / den
        s10 = s[1, 1] * t[1, 0] * s00 + s[1, 0]
        s11 = s[1, 1] * t[1, 0] * s01 + s[1, 1] * t[1, 1]
        s = np.array([[s00, s01], [s10, s11]])
    return s


def response_matrix_scalar(pol, layer_d, layer_n, kpar, omega, fromlayer, tolayer):
    """smuthi/layers.py:336-380 for one in-plane wavenumber."""
    layer_d = list(layer_d)
    layer_n = list(layer_n)
    if fromlayer == 0:
        s = scattering_matrix(pol, layer_d, layer_n, kpar, omega)
        lmat = np.array([[0, 0], [s[1, 0], 0]])
    elif fromlayer == len(layer_d) - 1:
        s = scattering_matrix(pol, layer_d, layer_n, kpar, omega)
        lmat = np.array([[0, s[0, 1]], [0, 0]])
    else:
        sa = scattering_matrix(pol, [0] + layer_d[fromlayer:], [layer_n[fromlayer]] + layer_n[fromlayer:],
                               kpar, omega)
        sb = scattering_matrix(pol, layer_d[:fromlayer] + [0], layer_n[:fromlayer] + [layer_n[fromlayer]],
                               kpar, omega)
        lmat = np.dot(np.linalg.inv(np.array([[1, -sb[0, 1]], [-sa[1, 0], 1]])),
                      np.array([[0, sb[0, 1]], [sa[1, 0], 0]]))
    if tolayer > fromlayer:
        tm = transfer_matrix(pol, layer_d[fromlayer:tolayer + 1], layer_n[fromlayer:tolayer + 1], kpar, omega)
        lmat = np.dot(np.linalg.inv(tm), lmat + np.array([[1, 0], [0, 0]]))
    elif tolayer < fromlayer:
        tm = transfer_matrix(pol, layer_d[tolayer:fromlayer + 1], layer_n[tolayer:fromlayer + 1], kpar, omega)
        lmat = np.dot(tm, lmat + np.array([[0, 0], [0, 1]]))
    return np.array(lmat, dtype=complex)


def response_matrix(pol, layer_d, layer_n, kpar, omega, fromlayer, tolayer):
    """smuthi/layers.py:336-358 -- (2, 2, len(kpar)) stack of response matrices."""
    kpar = np.atleast_1d(kpar)
    out = np.zeros((2, 2, len(kpar)), dtype=complex)
    for i, kp in enumerate(kpar):
        out[:, :, i] = response_matrix_scalar(pol, layer_d, layer_n, kp, omega, fromlayer, tolayer)
    return out
