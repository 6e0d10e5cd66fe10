"""Oracle: lookup matvec, T-matrix apply, master operator and GMRES.

Restates ``CouplingMatrixRadialLookupCPU`` (smuthi/linearsystem/linear_system.py:903-975),
``TMatrix`` (:410-438), ``MasterMatrix`` (:388-407) and the GMRES branch of
``LinearSystem.solve`` (:254-286). Test infrastructure only.
"""
import numpy as np
import scipy.interpolate
import scipy.sparse.linalg

from .special import blocksize, index_triples, multi_to_single_index


def system_layout(particle_list):
    """Per-unknown (particle, lookup n, m) arrays and per-particle offsets.

    smuthi/linearsystem/linear_system.py:347-385 (SystemMatrix.index_block /
    index) and :934-949 (the per-n index lists of the CPU lookup class).
    """
    l_max = max(p.l_max for p in particle_list)
    m_max = max(p.m_max for p in particle_list)
    part, nlook, mm, offs = [], [], [], [0]
    for i, p in enumerate(particle_list):
        for (tau, l, m) in index_triples(p.l_max, p.m_max):
            part.append(i)
            nlook.append(multi_to_single_index(tau, l, m, l_max, m_max))
            mm.append(m)
        offs.append(offs[-1] + blocksize(p.l_max, p.m_max))
    return np.array(part), np.array(nlook), np.array(mm), np.array(offs)


class RadialLookupCPU:
    """CPU lookup coupling matrix, smuthi/linearsystem/linear_system.py:903-975.

    ``kind`` is 'linear' or 'cubic' (scipy ``interp1d``; cubic = not-a-knot
    spline) or 'cubic_hermite' (the 4-tap formula of the reference CUDA
    kernel, smuthi/linearsystem/linear_system_cuda.py:348-353, evaluated in
    float64 here).
    """

    def __init__(self, particle_list, table, rho_grid, kind='linear'):
        xy = np.array([p.position[:2] for p in particle_list], dtype=float)
        self.rho = np.sqrt((xy[:, None, 0] - xy[None, :, 0]) ** 2 + (xy[:, None, 1] - xy[None, :, 1]) ** 2)
        self.phi = np.arctan2(xy[:, None, 1] - xy[None, :, 1], xy[:, None, 0] - xy[None, :, 0])
        self.part, self.nlook, self.m, self.offs = system_layout(particle_list)
        self.bs = table.shape[1]
        self.shape = (len(self.part), len(self.part))
        self.table = table
        self.grid = rho_grid
        self.kind = kind
        self.sel = [np.where(self.nlook == n)[0] for n in range(self.bs)]
        self.m_of = np.zeros(self.bs, int)
        for n in range(self.bs):
            if len(self.sel[n]):
                self.m_of[n] = self.m[self.sel[n][0]]
        if kind in ('linear', 'cubic'):
            self.interp = [[scipy.interpolate.interp1d(rho_grid, table[:, a, b], kind=kind, axis=-1,
                                                       assume_sorted=True)
                            for b in range(self.bs)] for a in range(self.bs)]

    def _eval(self, a, b, r):
        if self.kind in ('linear', 'cubic'):
            return self.interp[a][b](r)
        h = self.grid[1] - self.grid[0]
        s = (r - self.grid[0]) / h
        k = np.floor(s).astype(int)
        w = s - np.floor(s)
        col = self.table[:, a, b]
        return ((-w ** 3 + 2 * w ** 2 - w) * col[k - 1] + (3 * w ** 3 - 5 * w ** 2 + 2) * col[k]
                + (-3 * w ** 3 + 4 * w ** 2 + w) * col[k + 1] + (w ** 3 - w ** 2) * col[k + 2]) / 2

    def matvec(self, x, rows=None):
        """y = W x (linear_system.py:958-973). ``rows`` restricts the output
        to the unknowns of the listed receiving particles (others stay 0)."""
        x = np.asarray(x)
        y = np.zeros(x.shape, complex)
        for n1 in range(self.bs):
            idx1 = self.sel[n1]
            if rows is not None:
                idx1 = idx1[np.isin(self.part[idx1], rows)]
            if len(idx1) == 0:
                continue
            i1 = self.part[idx1]
            for n2 in range(self.bs):
                idx2 = self.sel[n2]
                if len(idx2) == 0:
                    continue
                i2 = self.part[idx2]
                r = self.rho[i1[:, None], i2[None, :]]
                ph = self.phi[i1[:, None], i2[None, :]]
                M = self._eval(n1, n2, r) * np.exp(1j * (self.m_of[n2] - self.m_of[n1]) * ph)
                y[idx1] += M.dot(x[idx2])
        return y

    def linear_operator(self):
        return scipy.sparse.linalg.LinearOperator(self.shape, matvec=self.matvec, dtype=complex)


def t_apply(t_blocks, offs, v):
    """TMatrix.apply_t_matrix (linear_system.py:420-424): block-diagonal T v."""
    out = np.zeros(v.shape, complex)
    for i, t in enumerate(t_blocks):
        out[offs[i]:offs[i + 1]] = t.dot(v[offs[i]:offs[i + 1]])
    return out


def right_hand_side(t_blocks, offs, a_blocks):
    """TMatrix.right_hand_side (linear_system.py:429-438): T_i a_i stacked."""
    return np.concatenate([t.dot(a) for t, a in zip(t_blocks, a_blocks)])


def master_matvec(coupling, t_blocks, offs, v):
    """MasterMatrix lookup branch (linear_system.py:402-407): v - T W v."""
    return v - t_apply(t_blocks, offs, coupling.matvec(v))


def gmres_solve(coupling, t_blocks, offs, rhs, tol, restart=None, maxiter=None):
    """LinearSystem.solve GMRES branch (linear_system.py:271-286).

    The reference calls ``gmres(M, rhs, rhs, tol=tol, callback=...)`` with
    scipy's defaults (restart 20, atol 0). Returns (solution, info, n_iter).
    """
    n = len(rhs)
    op = scipy.sparse.linalg.LinearOperator((n, n), matvec=lambda v: master_matvec(coupling, t_blocks, offs, v),
                                            dtype=complex)
    count = [0]

    def cb(rk):
        count[0] += 1

    kw = dict(rtol=tol, atol=0.0, callback=cb, callback_type='legacy')
    if restart is not None:
        kw['restart'] = restart
    if maxiter is not None:
        kw['maxiter'] = maxiter
    x, info = scipy.sparse.linalg.gmres(op, rhs, rhs, **kw)
    return x, info, count[0]
