"""Newton's method, pseudo-arclength continuation and theta-method time
stepping over any backend that honours TransiFlow's interface contract
(``rhs``, ``jacobian``, ``solve``, ``mass_matrix``, ``set_parameter``).

The public classes take the constructor keywords and offer the methods of
the reference drivers (``transiflow/Continuation.py:47-482``,
``transiflow/TimeIntegration.py:29-115``), so scripts written for those run
here too.  The numerics are Keller's pseudo-arclength method as Seydel
states it (predictor 2.2.3, tangent 2.2.4-2.2.7, corrector 2.2.8-2.2.13),
with the reference's choices for what the method leaves open: a forward
difference of step ``delta`` for F_mu, the weight ``zeta = 1/N`` of the
state in the arclength norm, the Newton-count step-size rule of
Seydel p. 188 and a secant approach onto the target.  Evaluating those
formulas in the same order makes a branch computed here follow the same
parameter values, step sizes and accept/reject decisions as the reference's
driver on the same backend (checked bit for bit against the reference in the
tests).

The organisation is this module's own: a step is a loop over attempts, each
attempt is a corrector run described by a :class:`CorrectorResult`, and a
branch is a loop over steps that ends by landing on the target.

Beyond the reference:

* ``predictor``: a callable ``(interface, x0, mu0, dx, dmu, ds)`` returning a
  proposed point ``(x, mu)``, a proposed point with its own step size
  ``(x, mu, ds')`` (the point is then corrected on the arclength sphere of
  radius ds'), or ``None``.  The learned surrogate of
  :mod:`transiflow_gb300.surrogate` plugs in here.  A proposal gets a
  corrector budget of ``learned_newton_iterations``; when the corrector does
  not converge within it, the same step is redone from the secant predictor
  with the full budget and the original step size.  Every accepted point is
  judged by the same corrector.
* ``step_size``: a callable ``(interface, ds, iterations, ds_min, ds_max)``
  returning the next step size, replacing the Newton-count rule after
  accepted steps (failed attempts always halve by that rule).
* ``log``: a callable receiving one dict per accepted point.
* ``stats``: counts of interface calls, points and predictor outcomes.

Vectors may be NumPy arrays or :class:`transiflow_gb300.vector.DeviceVector`.
"""

import math
import time

__all__ = ['Continuation', 'TimeIntegration', 'CorrectorResult', 'dot', 'norm']


def dot(x, y):
    """Inner product that works for NumPy arrays and device vectors."""
    try:
        return x.T.conj() @ y
    except AttributeError:
        return x.dot(y)


def norm(x):
    """Euclidean norm, ``sqrt(|x . x|)``."""
    return math.sqrt(abs(dot(x, x)))


class CorrectorResult:
    """Outcome of one corrector run.

    ``converged`` is False when the run used its whole iteration budget or
    saw the residual grow; ``x``/``mu`` are then the starting point."""

    __slots__ = ('converged', 'x', 'mu', 'iterations', 'fnorm')

    def __init__(self, converged, x, mu, iterations, fnorm):
        self.converged = converged
        self.x = x
        self.mu = mu
        self.iterations = iterations
        self.fnorm = fnorm


class _Calls:
    """Interface calls with counters."""

    def __init__(self, interface, stats):
        self.itf = interface
        self.stats = stats

    def rhs(self, x):
        self.stats['rhs'] += 1
        return self.itf.rhs(x)

    def jacobian(self, x):
        self.stats['jacobian'] += 1
        return self.itf.jacobian(x)

    def solve(self, jac, *args):
        self.stats['solve'] += 1
        return self.itf.solve(jac, *args)

    def at(self, name, value):
        self.itf.set_parameter(name, value)


class Continuation:
    """Pseudo-arclength continuation of the steady states of an interface.

    Keywords as in ``transiflow.Continuation``: ``delta`` (finite-difference
    step of F_mu), ``destination_tolerance`` (how close to the target the
    branch must end), ``newton_tolerance``, ``maximum_newton_iterations``,
    ``optimal_newton_iterations`` (the step-size rule aims at this many
    corrector iterations), ``residual_check`` ('F': stop on ||F||, 'dx': stop
    on ||dx||), ``bordered_solver`` (solve the extended system in one call of
    ``interface.solve``) and ``verbose``.  Bifurcation detection and branch
    switching are not provided.
    """

    def __init__(self, interface, delta=1.0, destination_tolerance=1e-4,
                 newton_tolerance=1e-4, maximum_newton_iterations=10,
                 optimal_newton_iterations=3, residual_check='F',
                 bordered_solver=False, verbose=False, predictor=None, log=None, quiet=False,
                 learned_newton_iterations=4, step_size=None):
        if residual_check not in ('F', 'dx'):
            raise ValueError("residual_check must be 'F' or 'dx'")
        self.interface = interface
        self.delta = delta
        self.destination_tolerance = destination_tolerance
        self.newton_tolerance = newton_tolerance
        self.maximum_newton_iterations = maximum_newton_iterations
        self.optimal_newton_iterations = optimal_newton_iterations
        self.residual_check = residual_check
        self.bordered_solver = bordered_solver
        self.verbose = verbose
        self.quiet = quiet
        self.predictor = predictor
        self.learned_newton_iterations = learned_newton_iterations
        self.step_size = step_size
        self.log = log
        self.zeta = None
        self.newton_iterations = 0
        self.stats = {'rhs': 0, 'jacobian': 0, 'solve': 0, 'points': 0,
                      'failed_correctors': 0, 'learned_accepted': 0, 'learned_rejected': 0}
        self._calls = _Calls(interface, self.stats)
        self._clock = None

    # -- output ------------------------------------------------------------------
    def _note(self, text):
        if not self.quiet:
            print(text, flush=True)

    # -- Newton's method at a fixed parameter -----------------------------------------
    def newton(self, x0, tol=1e-10):
        """Newton's method for F(x) = 0 at the current parameters, from x0.
        Stops when ||F|| (or ||dx|| with residual_check='dx') drops below tol
        or after maximum_newton_iterations; returns the last iterate."""
        c = self._calls
        on_f = self.residual_check == 'F'
        x = x0
        it = 0
        for it in range(self.maximum_newton_iterations):
            f = c.rhs(x)
            fn = norm(f) if (on_f or self.verbose) else None
            if on_f and fn < tol:
                self._note('newton: ||F|| = %e after %d iterations' % (fn, it))
                break
            step = c.solve(c.jacobian(x), -f)
            x = x + step
            sn = norm(step) if (not on_f or self.verbose) else None
            if not on_f and sn < tol:
                self._note('newton: ||dx|| = %e after %d iterations' % (sn, it))
                break
            if self.verbose:
                self._note('newton: iteration %d, ||F|| = %e, ||dx|| = %e' % (it, fn, sn))
        self.newton_iterations = it
        return x

    # -- the extended (arclength) system -------------------------------------------------
    def _arclength_residual(self, diff, mu, mu0, ds):
        """r = zeta |x - x0|^2 + (1 - zeta) (mu - mu0)^2 - ds^2 (Seydel 2.2.8)."""
        z = self.zeta
        return z * diff.dot(diff) + (1 - z) * (mu - mu0) ** 2 - ds ** 2

    def _newton_update(self, name, x, mu, x0, mu0, f, ds):
        """One Newton update (dx, dmu) of the extended system at (x, mu)."""
        c = self._calls
        z = self.zeta
        diff = x - x0
        r = self._arclength_residual(diff, mu, mu0, ds)
        # F_mu by a forward difference (left-hand side of 2.2.9)
        c.at(name, mu + self.delta)
        f_mu = (c.rhs(x) - f) / self.delta
        c.at(name, mu)
        jac = c.jacobian(x)
        if self.bordered_solver:
            return c.solve(jac, -f, -r, f_mu, 2 * z * diff, 2 * (1 - z) * (mu - mu0))
        # two solves with F_x and the Schur complement in mu (2.2.12, 2.2.13)
        y_f = c.solve(jac, -f)
        y_mu = c.solve(jac, f_mu)
        dmu = (-r - 2 * z * diff.dot(y_f)) / (2 * (1 - z) * (mu - mu0) - 2 * z * diff.dot(y_mu))
        return y_f - dmu * y_mu, dmu

    def correct(self, name, x, mu, x0, mu0, ds, budget=None):
        """Run the corrector from the predicted point (x, mu) on the arclength
        sphere of radius ds around (x0, mu0).  ``x`` is updated in place.

        The run stops successfully when ||F|| < newton_tolerance (or ||dx||
        with residual_check='dx'); it fails when the monitored norm grows from
        one iteration to the next or when the budget (default
        maximum_newton_iterations) is used up."""
        budget = self.maximum_newton_iterations if budget is None else budget
        c = self._calls
        on_f = self.residual_check == 'F'
        tol = self.newton_tolerance
        updates = 0
        fn = sn = None
        grew = False
        for it in range(budget):
            c.at(name, mu)
            f = c.rhs(x)
            if on_f or self.verbose:
                last_fn, fn = fn, norm(f)
            if on_f:
                if fn < tol:
                    self._note('corrector: ||F|| = %e after %d iterations' % (fn, it))
                    break
                if last_fn is not None and last_fn < fn:
                    grew = True
                    break
            dx, dmu = self._newton_update(name, x, mu, x0, mu0, f, ds)
            x += dx
            mu += dmu
            updates += 1
            if not on_f or self.verbose:
                last_sn, sn = sn, norm(dx)
            if not on_f and sn < tol:
                self._note('corrector: ||dx|| = %e after %d iterations' % (sn, it))
                break
            if self.verbose:
                self._note('corrector: iteration %d, ||F|| = %e, ||dx|| = %e' % (it, fn, sn))
            if not on_f and last_sn is not None and last_sn < sn:
                grew = True
                break
        # a run that used its whole budget counts as not converged, even when
        # its last update met the tolerance
        if grew or updates == budget:
            self.newton_iterations = budget
            self._note('corrector: no convergence, the step will be retried with a smaller ds')
            return CorrectorResult(False, x0, mu0, budget, fn)
        self.newton_iterations = updates
        c.at(name, mu)
        return CorrectorResult(True, x, mu, updates, fn)

    # -- step size ----------------------------------------------------------------------
    def _rescaled(self, ds, iterations, ds_min, ds_max):
        """Seydel's rule: scale ds by optimal/actual corrector iterations,
        within [1/2, 2], and clamp |ds| to [ds_min, ds_max]."""
        ratio = min(max(self.optimal_newton_iterations / max(iterations, 1), 0.5), 2.0)
        ds *= ratio
        ds = math.copysign(min(max(abs(ds), ds_min), ds_max), ds)
        if self.verbose:
            self._note('step size: ds = %e (x%e)' % (ds, ratio))
        return ds

    def _next_step_size(self, ds, ds_min, ds_max):
        if self.step_size is not None:
            return self.step_size(self.interface, ds, self.newton_iterations, ds_min, ds_max)
        return self._rescaled(ds, self.newton_iterations, ds_min, ds_max)

    # -- one step along the branch ------------------------------------------------------
    def _attempt(self, name, x0, mu0, dx, dmu, ds, proposal):
        if proposal is not None:
            x, mu = proposal[0], proposal[1]
            return self.correct(name, x, mu, x0, mu0, ds, self.learned_newton_iterations)
        return self.correct(name, x0 + ds * dx, mu0 + ds * dmu, x0, mu0, ds)

    def _advance(self, name, x0, mu0, dx, dmu, ds, ds_min, ds_max, learned):
        """Take one step from (x0, mu0) along the tangent (dx, dmu); retries
        with a reduced step size until the corrector converges.  Returns the
        new point, the secant tangent through it and the step size used."""
        proposal = None
        if learned and self.predictor is not None:
            proposal = self.predictor(self.interface, x0, mu0, dx, dmu, ds)
        secant_ds = ds
        while True:
            step = ds
            if proposal is not None and len(proposal) > 2:
                step = math.copysign(min(max(abs(proposal[2]), ds_min), ds_max), ds)
            res = self._attempt(name, x0, mu0, dx, dmu, step, proposal)
            # a corrected point must have moved in the parameter: the secant
            # tangent below divides by that change
            ok = res.converged and res.mu != mu0
            if proposal is not None:
                proposal = None
                if ok:
                    self.stats['learned_accepted'] += 1
                    ds = step
                else:
                    # redo the same step from the secant predictor
                    self.stats['learned_rejected'] += 1
                    ds = secant_ds
                    continue
            if ok:
                break
            self.stats['failed_correctors'] += 1
            smaller = self._rescaled(ds, self.newton_iterations, ds_min, ds_max)
            if smaller == ds:
                raise Exception('continuation stalled: the corrector does not converge at the minimum step size')
            ds = smaller
        x, mu = res.x, res.mu
        self._note('%s: %f' % (name, mu))
        self.stats['points'] += 1
        if self.log is not None:
            self.log({'mu': mu, 'fnorm': res.fnorm, 'newton_iterations': res.iterations, 'ds': ds,
                      'wall_s': time.perf_counter() - (self._clock or time.perf_counter())})
        # secant tangent through the two points, per unit arclength (2.2.4)
        dmu_new = mu - mu0
        dx_new = x - x0
        if abs(dmu_new) < 1e-12:
            raise Exception('continuation stalled: parameter change below 1e-12')
        dx_new /= ds
        dmu_new /= ds
        return x, mu, dx_new, dmu_new, ds

    def _land(self, name, x, mu, dx, dmu, target, ds, ds_min, ds_max, maxit):
        """Secant steps onto mu = target once the branch has passed it."""
        for _ in range(maxit):
            if abs(target - mu) < self.destination_tolerance:
                self._calls.at(name, target)
                self._note('reached %s = %f' % (name, mu))
                break
            ds = 1 / dmu * (target - mu)
            x, mu, dx, dmu, ds = self._advance(name, x, mu, dx, dmu, ds, ds_min, ds_max, False)
        return x, mu

    def _first_tangent(self, name, x, mu):
        """Tangent at the starting point from F_x dx = -F_mu, dmu = 1,
        normalised in the arclength norm (2.2.5-2.2.7)."""
        c = self._calls
        c.at(name, mu + self.delta)
        f_up = c.rhs(x)
        c.at(name, mu)
        f = c.rhs(x)
        f_mu = (f_up - f) / self.delta
        dx = c.solve(c.jacobian(x), -f_mu)
        dmu = 1
        scale = math.sqrt(self.zeta * dx.dot(dx) + dmu ** 2)
        dmu /= scale
        dx /= scale
        return dx, dmu

    # -- a branch ----------------------------------------------------------------------
    def continuation(self, x0, parameter_name, start, target, ds, ds_min=0.01, ds_max=1000,
                     dx=None, dmu=None, maxit=1000, detect_bifurcations=False,
                     switch_branches=False, return_step=False, callback=None):
        """Follow the branch through (x0, start) in ``parameter_name`` until
        it reaches ``target``; returns the final (x, mu), plus the last step
        (dx*ds, dmu*ds) with return_step=True.  ``dx``/``dmu`` give the
        initial direction (a step, as returned with return_step), otherwise
        the tangent is computed; ``callback(interface, x, mu)`` is called
        before every step and at the end."""
        if detect_bifurcations or switch_branches:
            raise NotImplementedError('bifurcation detection and branch switching are not provided')
        self._clock = time.perf_counter()
        name = parameter_name
        x, mu = x0, start
        self.zeta = 1 / x.size
        if dx is None or dmu is None:
            dx, dmu = self._first_tangent(name, x, mu)
        else:
            dx = dx / ds
            dmu = dmu / ds
        for j in range(maxit):
            mu_prev = mu
            if callback is not None:
                callback(self.interface, x, mu)
            x, mu, dx, dmu, ds = self._advance(name, x, mu, dx, dmu, ds, ds_min, ds_max, True)
            if (mu_prev < target <= mu) or (mu_prev > target >= mu):
                x, mu = self._land(name, x, mu, dx, dmu, target, ds, ds_min, ds_max, maxit - j)
                break
            ds = self._next_step_size(ds, ds_min, ds_max)
        if callback is not None:
            callback(self.interface, x, mu)
        if return_step:
            return x, mu, dx * ds, dmu * ds
        return x, mu


class TimeIntegration:
    """Implicit theta-method time stepping, each step solved by Newton's
    method: M (x_n - x) / (theta dt) + F(x) + (1 - theta)/theta F(x_n) = 0,
    with Jacobian J(x) - M / (theta dt).  Keywords as in
    ``transiflow.TimeIntegration``."""

    def __init__(self, interface, theta=1.0, newton_tolerance=1e-10,
                 maximum_newton_iterations=10, residual_check='F', verbose=False, quiet=False):
        self.interface = interface
        self.theta = theta
        self.newton_tolerance = newton_tolerance
        self.maximum_newton_iterations = maximum_newton_iterations
        self.residual_check = residual_check
        self.verbose = verbose
        self.quiet = quiet

    def _note(self, text):
        if not self.quiet:
            print(text, flush=True)

    def _implicit_step(self, x_old, dt):
        itf = self.interface
        on_f = self.residual_check == 'F'
        theta = self.theta
        f_old = itf.rhs(x_old)
        mass = itf.mass_matrix()
        x = x_old
        for it in range(self.maximum_newton_iterations):
            g = mass @ (x_old - x) + dt * theta * itf.rhs(x) + dt * (1 - theta) * f_old
            g /= theta * dt
            gn = norm(g) if (on_f or self.verbose) else None
            if on_f and gn < self.newton_tolerance:
                self._note('time step: ||G|| = %e after %d Newton iterations' % (gn, it))
                break
            step = itf.solve(itf.jacobian(x) - mass / (theta * dt), -g)
            x = x + step
            sn = norm(step) if (not on_f or self.verbose) else None
            if not on_f and sn < self.newton_tolerance:
                self._note('time step: ||dx|| = %e after %d Newton iterations' % (sn, it))
                break
            if self.verbose:
                self._note('time step: iteration %d, ||G|| = %e, ||dx|| = %e' % (it, gn, sn))
        return x

    def integration(self, x0, dt, tmax, callback=None):
        """Steps of size dt from t = 0 until t >= tmax; returns (x, t).
        ``callback(interface, x, t)`` is called at the start and after every
        step."""
        x, t = x0, 0
        if callback:
            callback(self.interface, x, t)
        while t < tmax:
            x = self._implicit_step(x, dt)
            t += dt
            self._note('t = %f' % t)
            if callback:
                callback(self.interface, x, t)
        return x, t
