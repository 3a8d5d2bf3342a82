"""Vectorised NumPy restatement of TransiFlow's finite-volume discretisation.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).

Every array operation below performs, element by element, the same IEEE
operations in the same order as the reference's per-cell Python loops, so the
atoms, the RHS and the CSR Jacobian agree with the reference bit for bit.
Where the reference evaluates ``a * b * 1 / 2`` the restatement keeps that
left-to-right order, and sums of atoms are taken in the reference's order.

Reference files (BIMAU/transiflow 1.0.1):
  transiflow/utils.py              coordinates, state layout
  transiflow/Discretization.py     linear/nonlinear atoms, assembly
  transiflow/BoundaryConditions.py boundary folding and forcing
  transiflow/CrsMatrix.py          compress (merge + 1e-14 drop)
"""

import numpy as np

DROP_TOL = 1e-14   # CrsMatrix.compress threshold, CrsMatrix.py:65


# ---------------------------------------------------------------------------
# Coordinates (utils.py:175-267, Discretization.py:186-208)
# ---------------------------------------------------------------------------

def uniform_coordinates(start, end, n):
    """utils.create_uniform_coordinate_vector, utils.py:175-197."""
    h = (end - start) / n
    return np.roll(start + np.arange(-1, n + 2) * h, -2)


def _fix_ghosts(c, start, end):
    # utils.py:225-231: the outer ghost cell mirrors the first/last cell.
    d = c[0] - c[-1]
    if start == 0:
        c[-2] = c[-1] - d
    if end == 1:
        c[-3] = c[-4] + d
    return c


def tanh_coordinates(start, end, n, sigma):
    """utils.create_stretched_coordinate_vector, utils.py:199-232."""
    u = uniform_coordinates(0, 1, n)
    u = 0.5 * (1 + np.tanh(2 * sigma * (u - 0.5)) / np.tanh(sigma))
    return _fix_ghosts(start + u * (end - start), start, end)


def sin_coordinates(start, end, n, sigma):
    """utils.create_stretched_coordinate_vector2, utils.py:234-267."""
    u = uniform_coordinates(0, 1, n)
    u = u - sigma * np.sin(2 * np.pi * u)
    return _fix_ghosts(start + u * (end - start), start, end)


def coordinate_vector(parameters, start, end, n):
    """Discretization.get_coordinate_vector, Discretization.py:186-208."""
    if parameters.get('Grid Stretching', False) or 'Grid Stretching Factor' in parameters:
        if parameters.get('Grid Stretching Method', 'tanh') == 'sin':
            return sin_coordinates(start, end, n, parameters.get('Grid Stretching Factor', 0.1))
        return tanh_coordinates(start, end, n, parameters.get('Grid Stretching Factor', 1.5))
    return uniform_coordinates(start, end, n)


class _Metric:
    """Per-axis spacings used by the stencil primitives.

    For cell index m along an axis with face coordinates ``c``:
      D  = c[m] - c[m-1]            Dp = c[m+1] - c[m]
      H  = (c[m] - c[m-2]) / 2      Hp = (c[m+1] - c[m-1]) / 2
      w0 = 1/2 * D / Hp             w1 = 1/2 * Dp / Hp
    (Discretization.py:740-1266 compute these scalars per cell.)
    """

    def __init__(self, c, n):
        m = np.arange(n)
        self.D = c[m] - c[m - 1]
        self.Dp = c[m + 1] - c[m]
        self.H = (c[m] - c[m - 2]) / 2
        self.Hp = (c[m + 1] - c[m - 1]) / 2
        self.w0 = 1 / 2 * self.D / self.Hp
        self.w1 = 1 / 2 * self.Dp / self.Hp


# ---------------------------------------------------------------------------
# State layout (utils.py:23-173)
# ---------------------------------------------------------------------------

def state_mtx(state, nx, ny, nz, dof):
    """utils.create_state_mtx: [i, j, k, d] view of the interleaved vector."""
    return np.asarray(state).reshape(nz, ny, nx, dof).transpose(2, 1, 0, 3)


def state_vec(mtx):
    """utils.create_state_vec: inverse of :func:`state_mtx`."""
    return np.ascontiguousarray(mtx.transpose(2, 1, 0, 3)).reshape(-1)


def padded_state(state, nx, ny, nz, dof, xper=False, yper=False, zper=False):
    """utils.create_padded_state_mtx, utils.py:62-133."""
    s = np.zeros((nx + 2, ny + 2, nz + 2, dof))
    s[1:nx + 1, 1:ny + 1, 1:nz + 1, :] = state_mtx(state, nx, ny, nz, dof)
    if xper:
        s[0] = s[nx]
        s[nx + 1] = s[1]
    else:
        s[nx, :, :, 0] = 0
    if yper:
        s[:, 0] = s[:, ny]
        s[:, ny + 1] = s[:, 1]
    else:
        s[:, ny, :, 1] = 0
    if zper:
        s[:, :, 0] = s[:, :, nz]
        s[:, :, nz + 1] = s[:, :, 1]
    else:
        s[:, :, nz, 2] = 0
    return s


# ---------------------------------------------------------------------------
# CSR container (CrsMatrix.py:10-71)
# ---------------------------------------------------------------------------

class Csr:
    """Compressed rows with sorted, merged columns and |v| > 1e-14 kept."""

    def __init__(self, begA, jcoA, coA):
        self.begA = begA
        self.jcoA = jcoA
        self.coA = coA

    @property
    def n(self):
        return len(self.begA) - 1

    @property
    def nnz(self):
        return int(self.begA[-1])

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.coA, self.jcoA, self.begA), shape=(self.n, self.n))


def compress_entries(rows, cols, vals, n):
    """Assemble (row, col, val) triples listed in the reference's config order.

    Entries with |v| <= 1e-14 are skipped (assemble_jacobian,
    Discretization.py:515), then each row's columns are sorted and duplicates
    summed in their original order before the final |sum| > 1e-14 drop
    (CrsMatrix.compress, CrsMatrix.py:52-71).
    """
    keep = np.abs(vals) > DROP_TOL
    rows, cols, vals = rows[keep], cols[keep], vals[keep]
    order = np.lexsort((cols, rows))      # stable: equal keys keep config order
    rows, cols, vals = rows[order], cols[order], vals[order]
    if len(rows):
        first = np.ones(len(rows), dtype=bool)
        first[1:] = (rows[1:] != rows[:-1]) | (cols[1:] != cols[:-1])
        starts = np.flatnonzero(first)
        lens = np.diff(np.append(starts, len(vals)))
        acc = np.zeros(len(starts))
        for m in range(int(lens.max())):     # left-to-right, as compress does
            sel = lens > m
            acc[sel] += vals[starts[sel] + m]
        vals = acc
        rows, cols = rows[starts], cols[starts]
        keep = np.abs(vals) > DROP_TOL
        rows, cols, vals = rows[keep], cols[keep], vals[keep]
    beg = np.zeros(n + 1, dtype=np.int64)
    np.add.at(beg, rows + 1, 1)
    return Csr(np.cumsum(beg), cols.astype(np.int64), vals.astype(np.float64))


# ---------------------------------------------------------------------------
# Boundary folding (BoundaryConditions.py:55-544)
# ---------------------------------------------------------------------------

def _ix(axis, cell, d1=slice(None), d2=slice(None), off=None):
    idx = [slice(None)] * 8
    idx[axis] = cell
    idx[3] = d1
    idx[4] = d2
    if off is not None:
        idx[5 + axis] = off
    return tuple(idx)


# The forcing component zeroed by the east/north/top walls: u, v and -- as in
# the reference (BoundaryConditions.py:131, 221) -- v again for the top wall.
_WALL_FRC_VAR = (0, 1, 1)


def apply_wall(atom, frc, axis, high, sign):
    """no_slip_* (sign=-1) and free_slip_* (sign=+1), BoundaryConditions.py:55-233."""
    n = atom.shape[axis]
    if high:
        b = n - 1
        if sign < 0:
            atom[_ix(axis, b, off=1)] -= atom[_ix(axis, b, off=2)]
        else:
            atom[_ix(axis, b, off=1)] += atom[_ix(axis, b, off=2)]
        atom[_ix(axis, b, d2=axis, off=1)] = 0
        atom[_ix(axis, b, d1=axis)] = 0
        atom[_ix(axis, b, off=2)] = 0
        centre = list(_ix(axis, b, d1=axis, d2=axis))
        centre[5] = centre[6] = centre[7] = 1
        atom[tuple(centre)] = -1
        atom[_ix(axis, n - 2, d1=axis, d2=axis, off=2)] = 0
        fidx = [slice(None)] * 4
        fidx[axis] = b
        fidx[3] = _WALL_FRC_VAR[axis]
        frc[tuple(fidx)] = 0
    else:
        atom[_ix(axis, 0, d2=axis, off=0)] = 0
        if sign < 0:
            atom[_ix(axis, 0, off=1)] -= atom[_ix(axis, 0, off=0)]
        else:
            atom[_ix(axis, 0, off=1)] += atom[_ix(axis, 0, off=0)]
        atom[_ix(axis, 0, off=0)] = 0


def apply_forcing(atom, frc, axis, high, var, fc, ac):
    """_constant_forcing_*, BoundaryConditions.py:471-544.  fc is a scalar or,
    as ``numpy.ones((n1 + 2, n2 + 2)) * value`` there, an array over the
    boundary's two other axes including their ghosts, read at
    [i + o1 - 1, j + o2 - 1] (index -1 meaning the last)."""
    n = atom.shape[axis]
    b = n - 1 if high else 0
    out = 2 if high else 0
    face = atom[_ix(axis, b, d1=var, d2=var, off=out)]     # cells(2) x offsets(2)
    acc = np.zeros(face.shape[:2])
    n1, n2 = face.shape[:2]
    if np.ndim(fc):
        V = np.ones((n1 + 2, n2 + 2)) * fc
        i1 = np.arange(n1)[:, None]
        i2 = np.arange(n2)[None, :]
    for o2 in range(3):          # the later offset axis is the outer loop
        for o1 in range(3):
            if np.ndim(fc):
                acc += face[:, :, o1, o2] * V[i1 + o1 - 1, i2 + o2 - 1]
            else:
                acc += face[:, :, o1, o2] * fc
    fidx = [slice(None)] * 4
    fidx[axis] = b
    fidx[3] = var
    frc[tuple(fidx)] += acc
    atom[_ix(axis, b, d2=var, off=1)] += ac * atom[_ix(axis, b, d2=var, off=out)]
    atom[_ix(axis, b, d2=var, off=out)] = 0


# ---------------------------------------------------------------------------
# Discretisation
# ---------------------------------------------------------------------------

def _b3(a):
    return a[:, None, None]


def _b3y(a):
    return a[None, :, None]


def _b3z(a):
    return a[None, None, :]


class Discretization:
    """Restatement of transiflow.Discretization for the built-in problem types
    'Lid-driven Cavity', 'Differentially Heated Cavity', 'Rayleigh-Benard' and
    'Rayleigh-Benard Perturbation' (Discretization.py:106-733)."""

    def __init__(self, parameters, nx, ny, nz=1, dim=None, dof=None, x=None, y=None, z=None):
        self.parameters = parameters
        self.nx, self.ny, self.nz = nx, ny, nz
        self.dim = dim if dim is not None else (3 if nz > 1 else 2)
        self.problem = self.get_parameter('Problem Type', 'Lid-driven Cavity').lower()
        if dof is None:
            dof = self.dim + 1
            if self.problem in ('rayleigh-benard', 'rayleigh-benard perturbation',
                                'differentially heated cavity'):
                dof = self.dim + 2
            elif self.problem == 'amoc':
                dof = self.dim + 3
        self.dof = dof
        if self.problem not in ('lid-driven cavity', 'differentially heated cavity',
                                'rayleigh-benard', 'rayleigh-benard perturbation', 'double gyre', 'amoc'):
            raise NotImplementedError('problem type %s' % self.problem)
        self.zper = nz == 1
        p = parameters
        self.x = coordinate_vector(p, p.get('X-min', 0.0), p.get('X-max', 1.0), nx) if x is None else np.asarray(x)
        self.y = coordinate_vector(p, p.get('Y-min', 0.0), p.get('Y-max', 1.0), ny) if y is None else np.asarray(y)
        self.z = coordinate_vector(p, p.get('Z-min', 0.0), p.get('Z-max', 1.0), nz) if z is None else np.asarray(z)
        self.X = _Metric(self.x, nx)
        self.Y = _Metric(self.y, ny)
        self.Z = _Metric(self.z, nz)

    def get_parameter(self, name, default=0):
        return self.parameters.get(name, default) if name in self.parameters else default

    def set_parameter(self, name, value):
        self.parameters[name] = value

    def _atom(self):
        return np.zeros((self.nx, self.ny, self.nz, self.dof, self.dof, 3, 3, 3))

    # -- linear primitives (Discretization.py:740-1099) -----------------------

    def _line(self, d1, d2, axis, vals):
        """Dense atom with values at offsets 0..2 along ``axis`` (others 1)."""
        a = self._atom()
        shape = (self.nx, self.ny, self.nz)
        for o, v in vals.items():
            off = [1, 1, 1]
            off[axis] = o
            a[:, :, :, d1, d2, off[0], off[1], off[2]] = np.broadcast_to(v, shape)
        return a

    def _second(self, d1, d2, axis, hlo, hhi, w1, w2):
        a0 = 1 / hlo * w1 * w2
        a2 = 1 / hhi * w1 * w2
        return self._line(d1, d2, axis, {0: a0, 1: -a0 - a2, 2: a2})

    def _geo(self):
        X, Y, Z = self.X, self.Y, self.Z
        return dict(Dx=_b3(X.D), Dpx=_b3(X.Dp), Hx=_b3(X.H), Hpx=_b3(X.Hp),
                    Dy=_b3y(Y.D), Dpy=_b3y(Y.Dp), Hy=_b3y(Y.H), Hpy=_b3y(Y.Hp),
                    Dz=_b3z(Z.D), Dpz=_b3z(Z.Dp), Hz=_b3z(Z.H), Hpz=_b3z(Z.Hp))

    def linear_part(self):
        """Discretization._linear_part_2D/_3D, Discretization.py:229-317."""
        g = self._geo()
        Dx, Dpx, Hx, Hpx = g['Dx'], g['Dpx'], g['Hx'], g['Hpx']
        Dy, Dpy, Hy, Hpy = g['Dy'], g['Dpy'], g['Hy'], g['Hpy']
        Dz, Dpz, Hz, Hpz = g['Dz'], g['Dpz'], g['Hz'], g['Hpz']
        dim, dof = self.dim, self.dof
        Re = self.get_parameter('Reynolds Number', 1.0)
        Ra = self.get_parameter('Rayleigh Number', 1.0)
        Pr = self.get_parameter('Prandtl Number', 1.0)
        Gr = self.get_parameter('Grashof Number', Ra / Pr)
        beta = self.get_parameter('Rossby Parameter')
        if beta and dim != 2:
            raise NotImplementedError('Coriolis term in 3D')
        if Re == 0:
            Re = 1
        if Gr == 0:
            Gr = 1 / Pr

        u_xx = self._second(0, 0, 0, Dx, Dpx, Dy, Dz)
        u_yy = self._second(0, 0, 1, Hy, Hpy, Hpx, Dz)
        v_xx = self._second(1, 1, 0, Hx, Hpx, Hpy, Dz)
        v_yy = self._second(1, 1, 1, Dy, Dpy, Dx, Dz)
        p_x = self._line(0, dim, 0, {1: -(Dy * Dz), 2: Dy * Dz})
        p_y = self._line(1, dim, 1, {1: -(Dx * Dz), 2: Dx * Dz})
        u_x = self._line(dim, 0, 0, {0: -(Dy * Dz), 1: Dy * Dz})
        v_y = self._line(dim, 1, 1, {0: -(Dx * Dz), 1: Dx * Dz})
        if dim == 2:
            atom = 1 / (Re * np.sqrt(Gr)) * (u_xx + u_yy + v_xx + v_yy) - (p_x + p_y) + (u_x + v_y)
            if beta:
                atom -= beta * self.coriolis()
            if dof > 3:
                T = dim + 1
                atom += 1 / (Pr * np.sqrt(Gr)) * (self._second(T, T, 0, Hx, Hpx, Dy, Dz)
                                                  + self._second(T, T, 1, Hy, Hpy, Dx, Dz))
                fa = Hpy * Dx * Dz / 2
                atom += self._line(1, T, 1, {1: fa, 2: fa})
            if dof > 4:
                Le = self.get_parameter('Lewis Number', 1.0)
                Sv = dim + 2
                atom += 1 / (Le * Pr * np.sqrt(Gr)) * (self._second(Sv, Sv, 0, Hx, Hpx, Dy, Dz)
                                                       + self._second(Sv, Sv, 1, Hy, Hpy, Dx, Dz))
                fa = Hpy * Dx * Dz / 2
                atom -= self._line(1, Sv, 1, {1: fa, 2: fa})
            if self.problem == 'rayleigh-benard perturbation':
                Bi = self.get_parameter('Biot Number')
                ba = Hpy * Dx * Dz / 2
                atom += Bi / (Bi + 1) * self._line(dim + 1, 1, 1, {0: ba, 1: ba})
            return atom

        u_zz = self._second(0, 0, 2, Hz, Hpz, Hpx, Dy)
        v_zz = self._second(1, 1, 2, Hz, Hpz, Hpy, Dx)
        w_xx = self._second(2, 2, 0, Hx, Hpx, Hpz, Dy)
        w_yy = self._second(2, 2, 1, Hy, Hpy, Hpz, Dx)
        w_zz = self._second(2, 2, 2, Dz, Dpz, Dy, Dx)
        p_z = self._line(2, dim, 2, {1: -(Dy * Dx), 2: Dy * Dx})
        w_z = self._line(dim, 2, 2, {0: -(Dy * Dx), 1: Dy * Dx})
        atom = 1 / (Re * np.sqrt(Gr)) * (u_xx + u_yy + u_zz + v_xx + v_yy + v_zz
                                         + w_xx + w_yy + w_zz) \
            - (p_x + p_y + p_z) + (u_x + v_y + w_z)
        if dof > 4:
            T = dim + 1
            atom += 1 / (Pr * np.sqrt(Gr)) * (self._second(T, T, 0, Hx, Hpx, Dy, Dz)
                                              + self._second(T, T, 1, Hy, Hpy, Dx, Dz)
                                              + self._second(T, T, 2, Hz, Hpz, Dy, Dx))
            if self.nz > 1:
                fa = Hpz * Dy * Dx / 2
                atom += self._line(2, T, 2, {1: fa, 2: fa})
            else:
                fa = Hpy * Dx * Dz / 2
                atom += self._line(1, T, 1, {1: fa, 2: fa})
        if dof > 5:
            Le = self.get_parameter('Lewis Number', 1.0)
            Sv = dim + 2
            atom += 1 / (Le * Pr * np.sqrt(Gr)) * (self._second(Sv, Sv, 0, Hx, Hpx, Dy, Dz)
                                                   + self._second(Sv, Sv, 1, Hy, Hpy, Dx, Dz)
                                                   + self._second(Sv, Sv, 2, Hz, Hpz, Dy, Dx))
            if self.nz > 1:
                fa = Hpz * Dy * Dx / 2
                atom -= self._line(2, Sv, 2, {1: fa, 2: fa})
            else:
                fa = Hpy * Dx * Dz / 2
                atom -= self._line(1, Sv, 1, {1: fa, 2: fa})
        if self.problem == 'rayleigh-benard perturbation':
            Bi = self.get_parameter('Biot Number')
            if self.nz > 1:
                ba = Hpz * Dy * Dx / 2
                atom += Bi / (Bi + 1) * self._line(dim + 1, 2, 2, {0: ba, 1: ba})
            else:
                ba = Hpy * Dx * Dz / 2
                atom += Bi / (Bi + 1) * self._line(dim + 1, 1, 1, {0: ba, 1: ba})
        return atom

    def coriolis(self):
        """Discretization.coriolis, Discretization.py:1086-1099: beta-plane
        Coriolis couplings, y v averaged to u points and y u to v points."""
        g = self._geo()
        yj = _b3y(self.y[:self.ny])
        yjm = _b3y(self.y[np.arange(self.ny) - 1])
        a = self._atom()
        shape = (self.nx, self.ny, self.nz)
        cv = (g['Hpy'] * g['Dx'] * g['Dz'] / 2) * (yj / 2)       # v row, u at x-1/0, y 0/+1
        cu = (g['Hpx'] * g['Dy'] * g['Dz'] / 2) * (-(yj + yjm) / 4)   # u row, v at x 0/+1, y -1/0
        for ox in (0, 1):
            for oy in (1, 2):
                a[:, :, :, 1, 0, ox, oy, 1] = np.broadcast_to(cv, shape)
        for ox in (1, 2):
            for oy in (0, 1):
                a[:, :, :, 0, 1, ox, oy, 1] = np.broadcast_to(cu, shape)
        return a

    def wind_stress(self):
        """Discretization.wind_stress, Discretization.py:1101-1118: zonal
        wind forcing of the u equation (not on the east wall)."""
        alpha = self.get_parameter('Wind Stress Parameter')
        asym = self.get_parameter('Asymmetry Parameter')
        frc = np.zeros((self.nx, self.ny, self.nz, self.dof))
        x, y, z = self.x, self.y, self.z
        i = np.arange(self.nx - 1)[:, None, None]
        j = np.arange(self.ny)[None, :, None]
        k = np.arange(self.nz)[None, None, :]
        dx = (x[i + 1] - x[i - 1]) / 2
        dy = y[j] - y[j - 1]
        dz = z[k] - z[k - 1]
        yc = (y[j] + y[j - 1]) / 2
        f = - (1 - asym) * np.cos(2 * np.pi * yc) - asym * np.cos(np.pi * yc)
        f = f * (alpha / (2 * np.pi) * dx * dy * dz)
        frc[:self.nx - 1, :, :, 0] = f
        return frc

    # -- nonlinear part (Discretization.py:319-365, 1178-1467) -----------------

    def nonlinear_part(self, state):
        nx, ny, nz, dim, dof = self.nx, self.ny, self.nz, self.dim, self.dof
        S = padded_state(state, nx, ny, nz, dof, False, False, self.zper)
        F = self._atom()
        J = self._atom()
        Re = self.get_parameter('Reynolds Number')
        if Re == 0 and not dof > dim + 1:
            return J, F
        X, Y, Z = self.X, self.Y, self.Z
        Dx, Dy, Dz = _b3(X.D), _b3y(Y.D), _b3z(Z.D)
        Hpx, Hpy, Hpz = _b3(X.Hp), _b3y(Y.Hp), _b3z(Z.Hp)
        w0x, w1x = _b3(X.w0), _b3(X.w1)
        w0y, w1y = _b3y(Y.w0), _b3y(Y.w1)
        w0z, w1z = _b3z(Z.w0), _b3z(Z.w1)

        def sub(A, d1, d2, o, v):
            A[:, :, :, d1, d2, o[0], o[1], o[2]] -= v

        def avg(Sd, axis):
            # average_x/y/z, Discretization.py:1178-1209
            if axis == 0:
                c = Sd[:, 1:ny + 1, 1:nz + 1]
                out = np.zeros((nx + 1, ny, nz))
                out += 1 / 2 * c[0:nx + 1]
                out += 1 / 2 * c[1:nx + 2]
            elif axis == 1:
                c = Sd[1:nx + 1, :, 1:nz + 1]
                out = np.zeros((nx, ny + 1, nz))
                out += 1 / 2 * c[:, 0:ny + 1]
                out += 1 / 2 * c[:, 1:ny + 2]
            else:
                c = Sd[1:nx + 1, 1:ny + 1, :]
                out = np.zeros((nx, ny, nz + 1))
                out += 1 / 2 * c[:, :, 0:nz + 1]
                out += 1 / 2 * c[:, :, 1:nz + 2]
            return out

        def wavg(Sd, axis):
            # weighted_average_x/y/z, Discretization.py:1211-1266
            if axis == 0:
                c = Sd[:, 0:ny + 1, 0:nz + 1]
                out = np.zeros((nx, ny + 1, nz + 1))
                out += w0x * c[1:nx + 1]
                out += w1x * c[2:nx + 2]
            elif axis == 1:
                c = Sd[0:nx + 1, :, 0:nz + 1]
                out = np.zeros((nx + 1, ny, nz + 1))
                out += w0y * c[:, 1:ny + 1]
                out += w1y * c[:, 2:ny + 2]
            else:
                c = Sd[0:nx + 1, 0:ny + 1, :]
                out = np.zeros((nx + 1, ny + 1, nz))
                out += w0z * c[:, :, 1:nz + 1]
                out += w1z * c[:, :, 2:nz + 2]
            return out

        def self_conv(var, axis, a2):
            # u_u_x / v_v_y / w_w_z: both F and J get the same four updates
            A = avg(S[..., var], axis)
            a1 = -a2
            lo = [slice(None)] * 3
            hi = [slice(None)] * 3
            lo[axis] = slice(0, A.shape[axis] - 1)
            hi[axis] = slice(1, A.shape[axis])
            t1 = a1 * A[tuple(lo)] * 1 / 2
            t2 = a2 * A[tuple(hi)] * 1 / 2
            for M in (F, J):
                for o, t in ((0, t1), (1, t1), (1, t2), (2, t2)):
                    off = [1, 1, 1]
                    off[axis] = o
                    sub(M, var, var, off, t)

        def cross(row, col, ax_row, ax_col, b1, Wrow, Acol, w0, w1, wsl_lo, wsl_hi, asl_lo, asl_hi):
            # u_v_x-type term: F part on (row,row) along ax_row, J part on (row,col)
            b0 = -b1
            tF0 = b0 * Wrow[wsl_lo] * 1 / 2
            tF1 = b1 * Wrow[wsl_hi] * 1 / 2
            for o, t in ((0, tF0), (1, tF0), (1, tF1), (2, tF1)):
                off = [1, 1, 1]
                off[ax_row] = o
                sub(F, row, row, off, t)
            p0 = b0 * Acol[asl_lo]
            p1 = b1 * Acol[asl_hi]
            for orow, p in ((0, p0), (1, p1)):
                for ocol, w in ((1, w0), (2, w1)):
                    sub(J, row, col, _cross_off(ax_row, ax_col, orow, ocol), p * w)

        S0, S1 = S[..., 0], S[..., 1]
        all_ = slice(None)
        # u_u_x, Discretization.py:1268-1279
        self_conv(0, 0, Dy * Dz)
        # u_v_x, Discretization.py:1281-1295 (v-row; J wrt u)
        cross(1, 0, 0, 1, Hpy * Dz, wavg(S0, 1), avg(S1, 0), w0y, w1y,
              (slice(0, nx), all_, slice(1, nz + 1)), (slice(1, nx + 1), all_, slice(1, nz + 1)),
              (slice(0, nx), all_, all_), (slice(1, nx + 1), all_, all_))
        # v_u_y, Discretization.py:1335-1349 (u-row; J wrt v)
        cross(0, 1, 1, 0, Hpx * Dz, wavg(S1, 0), avg(S0, 1), w0x, w1x,
              (all_, slice(0, ny), slice(1, nz + 1)), (all_, slice(1, ny + 1), slice(1, nz + 1)),
              (all_, slice(0, ny), all_), (all_, slice(1, ny + 1), all_))
        # v_v_y, Discretization.py:1351-1362
        self_conv(1, 1, Dx * Dz)
        if dim > 2:
            S2 = S[..., 2]
            # u_w_x, Discretization.py:1297-1311 (w-row; J wrt u)
            cross(2, 0, 0, 2, Hpz * Dy, wavg(S0, 2), avg(S2, 0), w0z, w1z,
                  (slice(0, nx), slice(1, ny + 1), all_), (slice(1, nx + 1), slice(1, ny + 1), all_),
                  (slice(0, nx), all_, all_), (slice(1, nx + 1), all_, all_))
            # v_w_y, Discretization.py:1364-1378 (w-row; J wrt v)
            cross(2, 1, 1, 2, Hpz * Dx, wavg(S1, 2), avg(S2, 1), w0z, w1z,
                  (slice(1, nx + 1), slice(0, ny), all_), (slice(1, nx + 1), slice(1, ny + 1), all_),
                  (all_, slice(0, ny), all_), (all_, slice(1, ny + 1), all_))
            # w_u_z, Discretization.py:1402-1416 (u-row; J wrt w)
            cross(0, 2, 2, 0, Hpx * Dy, wavg(S2, 0), avg(S0, 2), w0x, w1x,
                  (all_, slice(1, ny + 1), slice(0, nz)), (all_, slice(1, ny + 1), slice(1, nz + 1)),
                  (all_, all_, slice(0, nz)), (all_, all_, slice(1, nz + 1)))
            # w_v_z, Discretization.py:1418-1432 (v-row; J wrt w)
            cross(1, 2, 2, 1, Hpy * Dx, wavg(S2, 1), avg(S1, 2), w0y, w1y,
                  (slice(1, nx + 1), all_, slice(0, nz)), (slice(1, nx + 1), all_, slice(1, nz + 1)),
                  (all_, all_, slice(0, nz)), (all_, all_, slice(1, nz + 1)))
            # w_w_z, Discretization.py:1434-1445
            self_conv(2, 2, Dy * Dx)
        if dof > dim + 1:
            T = dim + 1
            ST = S[..., T]
            # u_C_x, Discretization.py:1313-1325
            self._scalar_conv(F, J, T, 0, Dy * Dz, S[0:nx + 1, 1:ny + 1, 1:nz + 1, 0], avg(ST, 0))
            # v_C_y, Discretization.py:1380-1392
            self._scalar_conv(F, J, T, 1, Dx * Dz, S[1:nx + 1, 0:ny + 1, 1:nz + 1, 1], avg(ST, 1))
            if dim > 2:
                # w_C_z, Discretization.py:1447-1459
                self._scalar_conv(F, J, T, 2, Dy * Dx, S[1:nx + 1, 1:ny + 1, 0:nz + 1, 2], avg(ST, 2))
        if dof > dim + 2:
            Sv = dim + 2
            SS = S[..., Sv]
            # u_S_x, v_S_y, w_S_z: u_C_x etc. for the salinity (Discretization.py:1331-1467)
            self._scalar_conv(F, J, Sv, 0, Dy * Dz, S[0:nx + 1, 1:ny + 1, 1:nz + 1, 0], avg(SS, 0))
            self._scalar_conv(F, J, Sv, 1, Dx * Dz, S[1:nx + 1, 0:ny + 1, 1:nz + 1, 1], avg(SS, 1))
            if dim > 2:
                self._scalar_conv(F, J, Sv, 2, Dy * Dx, S[1:nx + 1, 1:ny + 1, 0:nz + 1, 2], avg(SS, 2))
        J += F
        return J, F

    @staticmethod
    def _scalar_conv(F, J, var, axis, q1, U, C):
        q0 = -q1
        n = U.shape[axis] - 1
        lo = [slice(None)] * 3
        hi = [slice(None)] * 3
        lo[axis] = slice(0, n)
        hi[axis] = slice(1, n + 1)
        lo, hi = tuple(lo), tuple(hi)
        tF0 = q0 * U[lo] * 1 / 2
        tF1 = q1 * U[hi] * 1 / 2
        for o, t in ((0, tF0), (1, tF0), (1, tF1), (2, tF1)):
            off = [1, 1, 1]
            off[axis] = o
            F[:, :, :, var, var, off[0], off[1], off[2]] -= t
        for o, t in ((0, q0 * C[lo]), (1, q1 * C[hi])):
            off = [1, 1, 1]
            off[axis] = o
            J[:, :, :, var, axis, off[0], off[1], off[2]] -= t

    # -- boundary conditions (Discretization.py:577-643) -----------------------

    def bc_program(self):
        """The built-in problems' boundary-condition call sequences as
        ('wall', axis, high, sign) / ('force', axis, high, var, fc, ac) ops."""
        dim, nz = self.dim, self.nz
        T = dim + 1
        ops = []

        def wall(axis, high, sign=-1):
            ops.append(('wall', axis, high, sign))

        def force(axis, high, var, fc, ac):
            ops.append(('force', axis, high, var, fc, ac))

        def lid(axis, high, vel):
            force(axis, high, 0, 2 * vel, -1)   # moving_lid_north/top force u
            wall(axis, high)

        def coord(axis):
            return (self.x, self.y, self.z)[axis], (self.nx, self.ny, self.nz)[axis]

        def heat_flux(axis, high, q, biot=0.0):
            c, n = coord(axis)
            if high:
                h = (c[n] - c[n - 2]) / 2
                force(axis, True, T, h * q / (1 + h * biot / 2), (1 - h * biot / 2) / (1 + h * biot / 2))
            else:
                h = (c[0] - c[-2]) / 2
                force(axis, False, T, -h * q / (1 - h * biot / 2), (1 + h * biot / 2) / (1 - h * biot / 2))

        def temperature(axis, high, t):
            force(axis, high, T, 2 * t, -1)

        p = self.problem
        if p == 'lid-driven cavity':
            v = self.get_parameter('Lid Velocity', 1)
            wall(0, True)
            wall(0, False)
            wall(1, False)
            if dim == 2 or nz <= 1:
                lid(1, True, v)
                return ops
            wall(1, True)
            wall(2, False)
            lid(2, True, v)
        elif p in ('rayleigh-benard', 'rayleigh-benard perturbation'):
            asym = self.get_parameter('Asymmetry Parameter')
            heat_flux(0, True, asym)
            heat_flux(0, False, 0)
            wall(0, True)
            wall(0, False)
            Bi = self.get_parameter('Biot Number')
            bottom = 1 if p == 'rayleigh-benard' else 0
            if dim == 2 or nz <= 1:
                heat_flux(1, True, 0, Bi)
                temperature(1, False, bottom)
                wall(1, True, +1)
                wall(1, False)
                return ops
            heat_flux(1, True, 0)
            heat_flux(1, False, 0)
            wall(1, True)
            wall(1, False)
            heat_flux(2, True, 0, Bi)
            temperature(2, False, bottom)
            wall(2, True, +1)
            wall(2, False)
        elif p == 'double gyre':
            wall(0, True)
            wall(0, False)
            wall(1, True, +1)
            wall(1, False, +1)
        elif p == 'amoc':
            # Discretization._amoc, Discretization.py:657-702
            Sv = dim + 2

            def salinity_flux(axis, high, q):
                c, n = coord(axis)
                if high:
                    force(axis, True, Sv, (c[n] - c[n - 2]) / 2 * q, 1)
                else:
                    force(axis, False, Sv, -((c[0] - c[-2]) / 2) * q, 1)

            heat_flux(0, True, 0)
            heat_flux(0, False, 0)
            salinity_flux(0, True, 0)
            salinity_flux(0, False, 0)
            wall(0, True, +1)
            wall(0, False, +1)
            heat_flux(1, False, 0)
            salinity_flux(1, False, 0)
            wall(1, False, +1)
            T_S, Q_S = self.amoc_profiles()
            theta = self.get_parameter('Temperature Forcing')
            sigma = self.get_parameter('Freshwater Flux')
            temperature(1, True, theta * T_S)
            salinity_flux(1, True, sigma * Q_S)
            wall(1, True, +1)
            ops.append(('pin', Sv))
        elif p == 'differentially heated cavity':
            temperature(0, True, -1 / 2)
            temperature(0, False, 1 / 2)
            wall(0, True)
            wall(0, False)
            heat_flux(1, True, 0)
            heat_flux(1, False, 0)
            wall(1, True)
            wall(1, False)
            if dim > 2 and nz > 1:
                heat_flux(2, True, 0)
                heat_flux(2, False, 0)
                wall(2, True)
                wall(2, False)
        return ops

    def boundaries(self, atom):
        """Discretization.boundaries, Discretization.py:704-714."""
        if self.problem == 'double gyre':
            frc = self.wind_stress()
        else:
            frc = np.zeros((self.nx, self.ny, self.nz, self.dof))
        for op in self.bc_program():
            if op[0] == 'wall':
                apply_wall(atom, frc, op[1], op[2], op[3])
            elif op[0] == 'pin':
                self.pin(atom, frc, op[1])
            else:
                apply_forcing(atom, frc, *op[1:])
        return state_vec(frc)

    def pin(self, atom, frc, var):
        """Fix one value of ``var`` (Discretization.py:690-702): every entry
        coupling to ``var`` of cell (0, 0, 0), periodic neighbours included,
        becomes 0, that row gets -1 on its diagonal and no forcing."""
        nx, ny, nz = self.nx, self.ny, self.nz
        i = np.arange(nx)[:, None, None, None, None, None]
        j = np.arange(ny)[None, :, None, None, None, None]
        k = np.arange(nz)[None, None, :, None, None, None]
        o = np.arange(3)
        x, y, z = o[None, None, None, :, None, None], o[None, None, None, None, :, None], \
            o[None, None, None, None, None, :]
        hit = (((i + x - 1) % nx) == 0) & (((j + y - 1) % ny) == 0) & (((k + z - 1) % nz) == 0)
        hit = np.broadcast_to(hit, (nx, ny, nz, 3, 3, 3))
        for d in range(self.dof):
            a = atom[:, :, :, d, var]
            a[hit] = 0
        atom[0, 0, 0, var, var, 1, 1, 1] = -1
        frc[0, 0, 0, var] = 0

    def amoc_profiles(self):
        """T_S and Q_S of Discretization._amoc (Discretization.py:674-689):
        surface temperature and salinity-flux profiles over the cell centres,
        shape (nx + 2, nz + 2), set in column 0."""
        c = self.x
        x = np.zeros(len(c) - 1)
        for m in range(-1, len(c) - 2):
            x[m] = (c[m] + c[m - 1]) / 2
        asym = self.get_parameter('Asymmetry Parameter')
        A = self.parameters.get('X-max', 1.0)
        T_S = np.zeros((self.nx + 2, self.nz + 2))
        T_S[:, 0] = 1 / 2 * ((1 - asym) * np.cos(2 * np.pi * (x / A - 1 / 2))
                             + asym * np.cos(np.pi * x / A) + 1)
        p = 2
        Q_S = np.zeros((self.nx + 2, self.nz + 2))
        Q_S[:, 0] = 3 * np.cos(p * np.pi * (x / A - 1 / 2)) - 6 / (p * np.pi) * np.sin(p * np.pi / 2)
        return T_S, Q_S

    # -- assembly (Discretization.py:367-548) ----------------------------------

    def assemble_rhs(self, state, atom):
        nx, ny, nz, dof = self.nx, self.ny, self.nz, self.dof
        S = padded_state(state, nx, ny, nz, dof, False, False, self.zper)
        out = np.zeros((nx, ny, nz, dof))
        for oz in range(3):
            for oy in range(3):
                for ox in range(3):
                    for d1 in range(dof):
                        for d2 in range(dof):
                            out[:, :, :, d1] += atom[:, :, :, d1, d2, ox, oy, oz] \
                                * S[ox:ox + nx, oy:oy + ny, oz:oz + nz, d2]
        return state_vec(out)

    def assemble_jacobian(self, atom):
        nx, ny, nz, dof = self.nx, self.ny, self.nz, self.dof
        n = nx * ny * nz * dof
        # rows in (k, j, i, d1) order, entries in config (d2, x, y, z) order
        vals = atom.transpose(2, 1, 0, 3, 4, 5, 6, 7).reshape(n, dof * 27)
        k, j, i, _, d2, ox, oy, oz = np.indices((nz, ny, nx, dof, dof, 3, 3, 3), sparse=True)
        cols = ((i + ox - 1) % nx) * dof + ((j + oy - 1) % ny) * nx * dof \
            + ((k + oz - 1) % nz) * nx * ny * dof + d2
        cols = np.broadcast_to(cols, (nz, ny, nx, dof, dof, 3, 3, 3)).reshape(n, dof * 27)
        rows = np.broadcast_to(np.arange(n)[:, None], (n, dof * 27))
        return compress_entries(rows.ravel(), cols.ravel(), vals.ravel(), n)

    def rhs(self, state):
        _, F = self.nonlinear_part(state)
        F += self.linear_part()
        frc = self.boundaries(F)
        return self.assemble_rhs(state, F) + frc

    def jacobian(self, state):
        J, _ = self.nonlinear_part(state)
        J += self.linear_part()
        self.boundaries(J)
        return self.assemble_jacobian(J)

    def mass_matrix(self):
        """Discretization.mass_matrix, Discretization.py:417-548 (diagonal)."""
        X, Y, Z = self.X, self.Y, self.Z
        Dx, Dy, Dz = _b3(X.D), _b3y(Y.D), _b3z(Z.D)
        Hpx, Hpy, Hpz = _b3(X.Hp), _b3y(Y.Hp), _b3z(Z.Hp)
        shape = (self.nx, self.ny, self.nz)
        m = np.zeros(shape + (self.dof,))
        m[..., 0] = np.broadcast_to(Hpx * Dy * Dz, shape)
        m[..., 1] = np.broadcast_to(Hpy * Dx * Dz, shape)
        if self.dim == 3:
            m[..., 2] = np.broadcast_to(Hpz * Dy * Dx, shape)
        if self.dof > self.dim + 1:
            m[..., self.dim + 1] = np.broadcast_to(Dx * Dy * Dz, shape)
        if self.dof > self.dim + 2:
            m[..., self.dim + 2] = np.broadcast_to(Dx * Dy * Dz, shape)
        diag = state_vec(m)
        n = len(diag)
        rows = np.arange(n)
        return compress_entries(rows, rows, diag, n)


def _cross_off(ax_row, ax_col, orow, ocol):
    off = [1, 1, 1]
    off[ax_row] = orow
    off[ax_col] = ocol
    return off
