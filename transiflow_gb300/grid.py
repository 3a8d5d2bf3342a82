"""Host-side description of a discretisation: coordinates, the per-axis
metric table uploaded to the GPU, the scalar coefficients and the boundary
program of the built-in problem types.

Everything here is O(nx + ny + nz) work done once per grid (coordinates,
metrics) or once per parameter change (scalars, boundary program) in
float64 NumPy, with the same formulas as the reference so the device
arithmetic sees bit-identical inputs:

  coordinates    transiflow/utils.py:175-267, Discretization.py:186-208
  scalars        Discretization._linear_part_2D/3D, Discretization.py:229-317
  boundaries     Discretization._lid_driven_cavity / _rayleigh_benard /
                 _differentially_heated_cavity, Discretization.py:577-643,
                 and BoundaryConditions.py:239-469 for the constants
"""

import numpy as np

from . import _lib

SUPPORTED_PROBLEMS = ('lid-driven cavity', 'differentially heated cavity',
                      'rayleigh-benard', 'rayleigh-benard perturbation')


def uniform_coordinates(start, end, n):
    """Faces of a uniform grid, rolled so that c[-1] is the low wall."""
    h = (end - start) / n
    return np.roll(start + np.arange(-1, n + 2) * h, -2)


def _mirror_ghosts(c, start, end):
    d = c[0] - c[-1]
    if start == 0:
        c[-2] = c[-1] - d
    if end == 1:
        c[-3] = c[-4] + d
    return c


def tanh_coordinates(start, end, n, sigma):
    u = uniform_coordinates(0, 1, n)
    u = 0.5 * (1 + np.tanh(2 * sigma * (u - 0.5)) / np.tanh(sigma))
    return _mirror_ghosts(start + u * (end - start), start, end)


def sin_coordinates(start, end, n, sigma):
    u = uniform_coordinates(0, 1, n)
    u = u - sigma * np.sin(2 * np.pi * u)
    return _mirror_ghosts(start + u * (end - start), start, end)


def coordinate_vector(parameters, start, end, n):
    if parameters.get('Grid Stretching', False) or 'Grid Stretching Factor' in parameters:
        if parameters.get('Grid Stretching Method', 'tanh') == 'sin':
            return sin_coordinates(start, end, n, parameters.get('Grid Stretching Factor', 0.1))
        return tanh_coordinates(start, end, n, parameters.get('Grid Stretching Factor', 1.5))
    return uniform_coordinates(start, end, n)


def metric_table(coords, sizes):
    """float64 [3, TF_METRIC_FIELDS, stride] table of per-axis spacings."""
    stride = max(sizes)
    t = np.zeros((3, _lib.TF_METRIC_FIELDS, stride))
    for a, (c, n) in enumerate(zip(coords, sizes)):
        c = np.asarray(c, dtype=np.float64)
        m = np.arange(n)
        D = c[m] - c[m - 1]
        Dp = c[m + 1] - c[m]
        H = (c[m] - c[m - 2]) / 2
        Hp = (c[m + 1] - c[m - 1]) / 2
        t[a, 0, :n] = D
        t[a, 1, :n] = Dp
        t[a, 2, :n] = H
        t[a, 3, :n] = Hp
        t[a, 4, :n] = 1 / D
        t[a, 5, :n] = 1 / Dp
        t[a, 6, :n] = 1 / H
        t[a, 7, :n] = 1 / Hp
        t[a, 8, :n] = 1 / 2 * D / Hp
        t[a, 9, :n] = 1 / 2 * Dp / Hp
    return t


def default_dof(parameters, dim):
    problem = parameters.get('Problem Type', 'Lid-driven Cavity').lower()
    if problem in ('rayleigh-benard', 'rayleigh-benard perturbation', 'differentially heated cavity'):
        return dim + 2
    if problem == 'amoc':
        return dim + 3
    return dim + 1


def get_parameter(parameters, name, default=0):
    return parameters.get(name, default) if name in parameters else default


class BoundaryProgram:
    """Records boundary-condition primitives in call order.

    It offers the method names of transiflow.BoundaryConditions for the
    primitives the GPU kernel implements, so the built-in problems -- and a
    user ``boundary_conditions(bc, atom)`` callback composed of these
    primitives -- translate into the op list the kernel replays per cell.
    """

    def __init__(self, nx, ny, nz, dim, dof, x, y, z):
        self.nx, self.ny, self.nz, self.dim, self.dof = nx, ny, nz, dim, dof
        self.x, self.y, self.z = x, y, z
        self.ops = []
        self.profiles = []

    # walls
    def _wall(self, axis, high, sign):
        self.ops.append((_lib.TF_BC_WALL, axis, int(high), sign, 0.0, 0.0))

    def _force(self, axis, high, var, fc, ac):
        if np.ndim(fc) != 0:
            # a forcing that varies along the face: numpy.ones((n1 + 2, n2 + 2))
            # * value as BoundaryConditions._constant_forcing broadcasts it;
            # in 2D only its column 0 (the centre of the second tangential
            # axis) multiplies nonzero entries
            if self.dim != 2 or axis > 1:
                raise NotImplementedError('varying boundary forcing is supported on 2D x/y faces only')
            n1 = self.ny if axis == 0 else self.nx
            n2 = self.nz
            prof = (np.ones((n1 + 2, n2 + 2)) * fc)[:, 0]
            self.ops.append((_lib.TF_BC_FORCE_PROFILE, axis, int(high), var, float(len(self.profiles)), float(ac)))
            self.profiles.append(np.ascontiguousarray(prof, dtype=np.float64))
            return
        self.ops.append((_lib.TF_BC_FORCE, axis, int(high), var, float(fc), float(ac)))

    def _pin(self, var):
        self.ops.append((_lib.TF_BC_PIN, 0, 0, var, 0.0, 0.0))

    def no_slip_east(self, atom=None): self._wall(0, True, -1)
    def no_slip_west(self, atom=None): self._wall(0, False, -1)
    def no_slip_north(self, atom=None): self._wall(1, True, -1)
    def no_slip_south(self, atom=None): self._wall(1, False, -1)
    def no_slip_top(self, atom=None): self._wall(2, True, -1)
    def no_slip_bottom(self, atom=None): self._wall(2, False, -1)
    def free_slip_east(self, atom=None): self._wall(0, True, 1)
    def free_slip_west(self, atom=None): self._wall(0, False, 1)
    def free_slip_north(self, atom=None): self._wall(1, True, 1)
    def free_slip_south(self, atom=None): self._wall(1, False, 1)
    def free_slip_top(self, atom=None): self._wall(2, True, 1)
    def free_slip_bottom(self, atom=None): self._wall(2, False, 1)

    # moving lids: forcing on the tangential component, then a no-slip wall
    def moving_lid_east(self, atom, velocity):
        self._force(0, True, 1, 2 * velocity, -1)
        self.no_slip_east()

    def moving_lid_west(self, atom, velocity):
        self._force(0, False, 1, 2 * velocity, -1)
        self.no_slip_west()

    def moving_lid_north(self, atom, velocity):
        self._force(1, True, 0, 2 * velocity, -1)
        self.no_slip_north()

    def moving_lid_south(self, atom, velocity):
        self._force(1, False, 0, 2 * velocity, -1)
        self.no_slip_south()

    def moving_lid_top(self, atom, velocity):
        self._force(2, True, 0, 2 * velocity, -1)
        self.no_slip_top()

    def moving_lid_bottom(self, atom, velocity):
        self._force(2, False, 0, 2 * velocity, -1)
        self.no_slip_bottom()

    # temperature and heat flux
    def _coord(self, axis):
        return ((self.x, self.nx), (self.y, self.ny), (self.z, self.nz))[axis]

    def _temperature(self, axis, high, t):
        self._force(axis, high, self.dim + 1, 2 * t, -1)

    def temperature_east(self, atom, t): self._temperature(0, True, t)
    def temperature_west(self, atom, t): self._temperature(0, False, t)
    def temperature_north(self, atom, t): self._temperature(1, True, t)
    def temperature_south(self, atom, t): self._temperature(1, False, t)
    def temperature_top(self, atom, t): self._temperature(2, True, t)
    def temperature_bottom(self, atom, t): self._temperature(2, False, t)

    def _heat_flux(self, axis, high, q, biot):
        c, n = self._coord(axis)
        if high:
            h = (c[n] - c[n - 2]) / 2
            self._force(axis, True, self.dim + 1, h * q / (1 + h * biot / 2),
                        (1 - h * biot / 2) / (1 + h * biot / 2))
        else:
            h = (c[0] - c[-2]) / 2
            self._force(axis, False, self.dim + 1, -h * q / (1 - h * biot / 2),
                        (1 + h * biot / 2) / (1 - h * biot / 2))

    def heat_flux_east(self, atom, q, biot=0.0): self._heat_flux(0, True, q, biot)
    def heat_flux_west(self, atom, q, biot=0.0): self._heat_flux(0, False, q, biot)
    def heat_flux_north(self, atom, q, biot=0.0): self._heat_flux(1, True, q, biot)
    def heat_flux_south(self, atom, q, biot=0.0): self._heat_flux(1, False, q, biot)
    def heat_flux_top(self, atom, q, biot=0.0): self._heat_flux(2, True, q, biot)
    def heat_flux_bottom(self, atom, q, biot=0.0): self._heat_flux(2, False, q, biot)

    # salinity flux (BoundaryConditions.py:423-469)
    def _salinity_flux(self, axis, high, q):
        c, n = self._coord(axis)
        if high:
            self._force(axis, True, self.dim + 2, (c[n] - c[n - 2]) / 2 * q, 1)
        else:
            self._force(axis, False, self.dim + 2, -((c[0] - c[-2]) / 2) * q, 1)

    def salinity_flux_east(self, atom, q): self._salinity_flux(0, True, q)
    def salinity_flux_west(self, atom, q): self._salinity_flux(0, False, q)
    def salinity_flux_north(self, atom, q): self._salinity_flux(1, True, q)
    def salinity_flux_south(self, atom, q): self._salinity_flux(1, False, q)
    def salinity_flux_top(self, atom, q): self._salinity_flux(2, True, q)
    def salinity_flux_bottom(self, atom, q): self._salinity_flux(2, False, q)

    def get_forcing(self):
        return None


def builtin_boundaries(parameters, bc, dim, nz):
    """The call sequences of Discretization._lid_driven_cavity,
    _rayleigh_benard, _differentially_heated_cavity, _double_gyre and _amoc
    (Discretization.py:577-702)."""
    problem = parameters.get('Problem Type', 'Lid-driven Cavity').lower()
    if problem == 'lid-driven cavity':
        v = get_parameter(parameters, 'Lid Velocity', 1)
        bc.no_slip_east()
        bc.no_slip_west()
        bc.no_slip_south()
        if dim == 2 or nz <= 1:
            bc.moving_lid_north(None, v)
            return
        bc.no_slip_north()
        bc.no_slip_bottom()
        bc.moving_lid_top(None, v)
    elif problem in ('rayleigh-benard', 'rayleigh-benard perturbation'):
        asym = get_parameter(parameters, 'Asymmetry Parameter')
        bc.heat_flux_east(None, asym)
        bc.heat_flux_west(None, 0)
        bc.no_slip_east()
        bc.no_slip_west()
        Bi = get_parameter(parameters, 'Biot Number')
        bottom = 1 if problem == 'rayleigh-benard' else 0
        if dim == 2 or nz <= 1:
            bc.heat_flux_north(None, 0, Bi)
            bc.temperature_south(None, bottom)
            bc.free_slip_north()
            bc.no_slip_south()
            return
        bc.heat_flux_north(None, 0)
        bc.heat_flux_south(None, 0)
        bc.no_slip_north()
        bc.no_slip_south()
        bc.heat_flux_top(None, 0, Bi)
        bc.temperature_bottom(None, bottom)
        bc.free_slip_top()
        bc.no_slip_bottom()
    elif problem == 'double gyre':
        # Discretization._double_gyre (Discretization.py:645-655); the wind
        # stress itself is a forcing of the kernel (tf_problem.wind)
        bc.no_slip_east()
        bc.no_slip_west()
        bc.free_slip_north()
        bc.free_slip_south()
    elif problem == 'amoc':
        # Discretization._amoc (Discretization.py:657-702)
        bc.heat_flux_east(None, 0)
        bc.heat_flux_west(None, 0)
        bc.salinity_flux_east(None, 0)
        bc.salinity_flux_west(None, 0)
        bc.free_slip_east()
        bc.free_slip_west()
        bc.heat_flux_south(None, 0)
        bc.salinity_flux_south(None, 0)
        bc.free_slip_south()
        T_S, Q_S = amoc_profiles(parameters, bc.x, bc.nx, bc.nz)
        bc.temperature_north(None, get_parameter(parameters, 'Temperature Forcing') * T_S)
        bc.salinity_flux_north(None, get_parameter(parameters, 'Freshwater Flux') * Q_S)
        bc.free_slip_north()
        bc._pin(dim + 2)
    elif problem == 'differentially heated cavity':
        bc.temperature_east(None, -1 / 2)
        bc.temperature_west(None, 1 / 2)
        bc.no_slip_east()
        bc.no_slip_west()
        bc.heat_flux_north(None, 0)
        bc.heat_flux_south(None, 0)
        bc.no_slip_north()
        bc.no_slip_south()
        if dim > 2 and nz > 1:
            bc.heat_flux_top(None, 0)
            bc.heat_flux_bottom(None, 0)
            bc.no_slip_top()
            bc.no_slip_bottom()
    else:
        raise NotImplementedError('problem type %r is not available on the GPU backend' % problem)


def scalars(parameters, dim, dof, nz):
    """Coefficients of the linear part, computed exactly as the reference."""
    Re = get_parameter(parameters, 'Reynolds Number', 1.0)
    Ra = get_parameter(parameters, 'Rayleigh Number', 1.0)
    Pr = get_parameter(parameters, 'Prandtl Number', 1.0)
    Gr = get_parameter(parameters, 'Grashof Number', Ra / Pr)
    rossby = get_parameter(parameters, 'Rossby Parameter')
    if rossby and dim != 2:
        raise NotImplementedError('the Coriolis term exists in 2D only (Discretization.py:253-255)')
    if dof > dim + 2 and dim != 2:
        raise NotImplementedError('salinity is compiled for 2D grids only')
    if Re == 0:
        Re = 1
    if Gr == 0:
        Gr = 1 / Pr
    visc = 1 / (Re * np.sqrt(Gr))
    cond = 1 / (Pr * np.sqrt(Gr))
    Le = get_parameter(parameters, 'Lewis Number', 1.0)
    sal = 1 / (Le * Pr * np.sqrt(Gr))
    nonlinear = not (get_parameter(parameters, 'Reynolds Number') == 0 and not dof > dim + 1)
    buoy_row = -1
    if dof > dim + 1:
        buoy_row = 2 if (dim == 3 and nz > 1) else 1
    biot_row, biot = -1, 0.0
    problem = parameters.get('Problem Type', 'Lid-driven Cavity').lower()
    if problem == 'rayleigh-benard perturbation':
        Bi = get_parameter(parameters, 'Biot Number')
        biot_row = 2 if (dim == 3 and nz > 1) else 1
        biot = Bi / (Bi + 1)
    wind = 0.0
    if problem == 'double gyre':
        wind = get_parameter(parameters, 'Wind Stress Parameter') / (2 * np.pi)
    return dict(visc=float(visc), cond=float(cond), nonlinear=int(nonlinear),
                buoy_row=buoy_row, biot_row=biot_row, biot=float(biot), rossby=float(rossby),
                wind=float(wind), asym=float(get_parameter(parameters, 'Asymmetry Parameter')), sal=float(sal))


def amoc_profiles(parameters, x, nx, nz):
    """T_S and Q_S of Discretization._amoc (Discretization.py:674-689) over
    the cell centres, shape (nx + 2, nz + 2), set in column 0."""
    xc = np.zeros(len(x) - 1)
    for m in range(-1, len(x) - 2):
        xc[m] = (x[m] + x[m - 1]) / 2
    asym = get_parameter(parameters, 'Asymmetry Parameter')
    A = parameters.get('X-max', 1.0)
    T_S = np.zeros((nx + 2, nz + 2))
    T_S[:, 0] = 1 / 2 * ((1 - asym) * np.cos(2 * np.pi * (xc / A - 1 / 2)) + asym * np.cos(np.pi * xc / A) + 1)
    p = 2
    Q_S = np.zeros((nx + 2, nz + 2))
    Q_S[:, 0] = 3 * np.cos(p * np.pi * (xc / A - 1 / 2)) - 6 / (p * np.pi) * np.sin(p * np.pi / 2)
    return T_S, Q_S


def aux_table(y, ny):
    """Per-row factors of the Coriolis term and the wind stress
    (Discretization.py:1086-1118), computed with the reference's operations:
    y[j]/2, -(y[j]+y[j-1])/4, cos(2 pi yc), cos(pi yc) for yc = (y[j]+y[j-1])/2."""
    j = np.arange(ny)
    yj, yjm = y[j], y[j - 1]
    yc = (yj + yjm) / 2
    return np.stack([yj / 2, -(yj + yjm) / 4, np.cos(2 * np.pi * yc), np.cos(np.pi * yc)])


def make_problem(parameters, nx, ny, nz, dim, dof, x, y, z, d_metric, stride, boundary_conditions=None,
                 d_aux=None, upload_profiles=None):
    """Fill the tf_problem structure for the current parameter values
    (d_aux: device copy of aux_table(y, ny), needed for the Coriolis term and
    the wind stress)."""
    sc = scalars(parameters, dim, dof, nz)
    bc = BoundaryProgram(nx, ny, nz, dim, dof, x, y, z)
    if boundary_conditions is None:
        builtin_boundaries(parameters, bc, dim, nz)
    else:
        boundary_conditions(bc, None)
    if len(bc.ops) > _lib.TF_MAX_BC_OPS:
        raise NotImplementedError('more than %d boundary operations' % _lib.TF_MAX_BC_OPS)
    p = _lib.Problem()
    p.nx, p.ny, p.nz, p.dim, p.dof = nx, ny, nz, dim, dof
    p.nonlinear = sc['nonlinear']
    p.buoy_row = sc['buoy_row']
    p.biot_row = sc['biot_row']
    p.visc, p.cond, p.biot = sc['visc'], sc['cond'], sc['biot']
    p.d_metric = d_metric
    p.metric_stride = stride
    p.nops = len(bc.ops)
    for t, (kind, axis, high, var, fc, ac) in enumerate(bc.ops):
        p.ops[t] = _lib.BcOp(kind, axis, high, var, fc, ac)
    p.rossby, p.wind, p.asym = sc['rossby'], sc['wind'], sc['asym']
    if (p.rossby or p.wind) and not d_aux:
        raise ValueError('the Coriolis term and the wind stress need the aux table')
    p.d_aux = d_aux
    p.sal = sc['sal']
    if bc.profiles:
        if upload_profiles is None:
            raise ValueError('varying boundary forcing needs a profile upload')
        table = np.stack(bc.profiles)
        p.d_prof = upload_profiles(table)
        p.prof_len = table.shape[1]
        p.nprof = table.shape[0]
    return p
