"""Newton, pseudo-arclength continuation and theta-method time integration.

These are the callers of the hot path.  They only talk to the backend through
the TransiFlow interface contract (``rhs``, ``jacobian``, ``solve``,
``mass_matrix``, ``set_parameter``) and reproduce the control flow and the
scalar arithmetic of the reference drivers, so a branch computed through the
``CUDA`` backend follows the same sequence of parameter values, step-size
adaptations and convergence decisions as one computed by the reference:

  Continuation     transiflow/Continuation.py:47-482
  TimeIntegration  transiflow/TimeIntegration.py:29-115

Vectors may be NumPy arrays or :class:`transiflow_gb300.vector.DeviceVector`;
both support ``x.size``, ``.dot``, ``.T.conj() @ y`` and scalar arithmetic.

Beyond the reference: an optional ``predictor`` callable can propose the
continuation predictor (the learned surrogate of
:mod:`transiflow_gb300.surrogate` plugs in here); the secant predictor of the
reference is used whenever it is absent or its corrector does not converge
within ``learned_newton_iterations`` iterations, and every accepted point is
judged by the same Newton corrector.  An
optional ``log`` callable receives one dict per accepted point.
"""

import math
import time

__all__ = ['Continuation', 'TimeIntegration', 'dot', 'norm']


def dot(x, y):
    """utils.dot, transiflow/utils.py:5-11."""
    try:
        return x.T.conj() @ y
    except AttributeError:
        return x.dot(y)


def norm(x):
    """utils.norm for vectors, transiflow/utils.py:13-21."""
    return math.sqrt(abs(dot(x, x)))


class Continuation:
    """Pseudo-arclength continuation with a Newton corrector.

    Same constructor keywords and defaults as transiflow.Continuation
    (Continuation.py:47-51).  Bifurcation detection needs eigenvalues, which
    the GPU backend does not provide; ``detect_bifurcations`` and
    ``switch_branches`` therefore raise NotImplementedError.
    """

    def __init__(self, interface, delta=1.0, destination_tolerance=1e-4,
                 newton_tolerance=1e-4, maximum_newton_iterations=10,
                 optimal_newton_iterations=3, residual_check='F',
                 bordered_solver=False, verbose=False, predictor=None, log=None, quiet=False,
                 learned_newton_iterations=4):
        self.interface = interface
        self.quiet = quiet
        self.verbose = verbose
        self.destination_tolerance = destination_tolerance
        self.delta = delta
        self.zeta = None
        self.maximum_newton_iterations = maximum_newton_iterations
        self.optimal_newton_iterations = optimal_newton_iterations
        self.newton_tolerance = newton_tolerance
        self.newton_iterations = 0
        self.residual_check = residual_check
        self.bordered_solver = bordered_solver
        self.predictor = predictor
        self.learned_newton_iterations = learned_newton_iterations
        self.log = log
        self.stats = {'rhs': 0, 'jacobian': 0, 'solve': 0, 'points': 0,
                      'failed_correctors': 0, 'learned_accepted': 0, 'learned_rejected': 0}
        self._t0 = None

    def _say(self, *args, **kwargs):
        """The reference's progress messages; quiet=True drops them (threads
        driving instances concurrently cannot redirect a shared stdout)."""
        if not self.quiet:
            print(*args, **kwargs)

    # -- counted interface calls ---------------------------------------------
    def _rhs(self, x):
        self.stats['rhs'] += 1
        return self.interface.rhs(x)

    def _jac(self, x):
        self.stats['jacobian'] += 1
        return self.interface.jacobian(x)

    def _solve(self, jac, *args):
        self.stats['solve'] += 1
        return self.interface.solve(jac, *args)

    # -- Newton (Continuation.py:67-114) --------------------------------------
    def newton(self, x0, tol=1e-10):
        x = x0
        k = 0
        for k in range(self.maximum_newton_iterations):
            fval = self._rhs(x)
            if self.residual_check == 'F' or self.verbose:
                fnorm = norm(fval)
            if self.residual_check == 'F' and fnorm < tol:
                self._say('Newton converged in %d iterations with ||F||=%e' % (k, fnorm), flush=True)
                break
            jac = self._jac(x)
            dx = self._solve(jac, -fval)
            x = x + dx
            if self.residual_check != 'F' or self.verbose:
                dxnorm = norm(dx)
            if self.residual_check != 'F' and dxnorm < tol:
                self._say('Newton converged in %d iterations with ||dx||=%e' % (k, dxnorm), flush=True)
                break
            if self.verbose:
                self._say('Newton status at iteration %d: ||F||=%e, ||dx||=%e' % (k, fnorm, dxnorm), flush=True)
        self.newton_iterations = k
        return x

    # -- corrector (Continuation.py:116-195) ----------------------------------
    def _newton_corrector(self, name, ds, x, x0, mu, mu0, maxit=None):
        maxit = self.maximum_newton_iterations if maxit is None else maxit
        self.newton_iterations = 0
        fnorm = None
        dxnorm = None
        self._last_fnorm = None
        for k in range(maxit):
            self.interface.set_parameter(name, mu)
            fval = self._rhs(x)
            if self.residual_check == 'F' or self.verbose:
                prev_norm = fnorm
                fnorm = norm(fval)
                self._last_fnorm = fnorm
            if self.residual_check == 'F' and fnorm < self.newton_tolerance:
                self._say('Newton corrector converged in %d iterations with ||F||=%e' % (k, fnorm), flush=True)
                break
            if self.residual_check == 'F' and prev_norm is not None and prev_norm < fnorm:
                self.newton_iterations = maxit
                break
            diff = x - x0
            rnp1 = self.zeta * diff.dot(diff) + (1 - self.zeta) * (mu - mu0) ** 2 - ds ** 2
            self.interface.set_parameter(name, mu + self.delta)
            dflval = (self._rhs(x) - fval) / self.delta
            self.interface.set_parameter(name, mu)
            jac = self._jac(x)
            if self.bordered_solver:
                dx, dmu = self._solve(jac, -fval, -rnp1, dflval, 2 * self.zeta * diff,
                                      2 * (1 - self.zeta) * (mu - mu0))
            else:
                z1 = self._solve(jac, -fval)
                z2 = self._solve(jac, dflval)
                dmu = (-rnp1 - 2 * self.zeta * diff.dot(z1)) / (2 * (1 - self.zeta) * (mu - mu0)
                                                                - 2 * self.zeta * diff.dot(z2))
                dx = z1 - dmu * z2
            x += dx
            mu += dmu
            self.newton_iterations += 1
            if self.residual_check != 'F' or self.verbose:
                prev_norm = dxnorm
                dxnorm = norm(dx)
            if self.residual_check != 'F' and dxnorm < self.newton_tolerance:
                self._say('Newton corrector converged in %d iterations with ||dx||=%e' % (k, dxnorm), flush=True)
                break
            if self.verbose:
                self._say('Newton corrector status at iteration %d: ||F||=%e, ||dx||=%e' % (k, fnorm, dxnorm), flush=True)
            if self.residual_check != 'F' and prev_norm is not None and prev_norm < dxnorm:
                self.newton_iterations = maxit
                break
        if self.newton_iterations == maxit:
            self._say('Newton did not converge. Adjusting step size and trying again', flush=True)
            self.stats['failed_correctors'] += 1
            return x0, mu0
        self.interface.set_parameter(name, mu)
        return x, mu

    # -- step-size control (Continuation.py:197-209) --------------------------
    def _adjust_step_size(self, ds, ds_min, ds_max):
        factor = self.optimal_newton_iterations / max(self.newton_iterations, 1)
        factor = min(max(factor, 0.5), 2.0)
        ds *= factor
        ds = math.copysign(min(max(abs(ds), ds_min), ds_max), ds)
        if self.verbose:
            self._say('New stepsize: ds=%e, factor=%e' % (ds, factor), flush=True)
        return ds

    # -- converge onto the target (Continuation.py:234-249) -------------------
    def _converge(self, name, x, mu, dx, dmu, target, ds, ds_min, ds_max, maxit):
        for _ in range(maxit):
            if abs(target - mu) < self.destination_tolerance:
                self.interface.set_parameter(name, target)
                self._say("Convergence achieved onto target %s = %f" % (name, mu), flush=True)
                break
            ds = 1 / dmu * (target - mu)
            x, mu, dx, dmu, ds = self._step(name, x, mu, dx, dmu, ds, ds_min, ds_max)
        return x, mu

    # -- one predictor/corrector step (Continuation.py:251-288) ---------------
    def _step(self, name, x, mu, dx, dmu, ds, ds_min, ds_max, use_predictor=False):
        mu0 = mu
        x0 = x
        learned = None
        if use_predictor and self.predictor is not None:
            learned = self.predictor(self.interface, x0, mu0, dx, dmu, ds)
        if learned is not None:
            x, mu = learned
        else:
            mu = mu0 + ds * dmu
            x = x0 + ds * dx
        x, mu = self._newton_corrector(name, ds, x, x0, mu, mu0,
                                       self.learned_newton_iterations if learned is not None else None)
        if learned is not None:
            if mu == mu0:
                # The learned predictor failed: fall back to the secant predictor.
                self.stats['learned_rejected'] += 1
                return self._step(name, x0, mu0, dx, dmu, ds, ds_min, ds_max)
            self.stats['learned_accepted'] += 1
        if mu == mu0:
            prev_ds = ds
            ds = self._adjust_step_size(ds, ds_min, ds_max)
            if prev_ds == ds:
                raise Exception('Newton cannot achieve convergence')
            return self._step(name, x0, mu0, dx, dmu, ds, ds_min, ds_max)
        self._say("%s: %f" % (name, mu), flush=True)
        self.stats['points'] += 1
        if self.log is not None:
            self.log({'mu': mu, 'fnorm': self._last_fnorm, 'newton_iterations': self.newton_iterations,
                      'ds': ds, 'wall_s': time.perf_counter() - (self._t0 or time.perf_counter())})
        dmu = mu - mu0
        dx = x - x0
        if abs(dmu) < 1e-12:
            raise Exception('dmu too small')
        dx /= ds
        dmu /= ds
        return x, mu, dx, dmu, ds

    # -- initial tangent (Continuation.py:330-350) ----------------------------
    def _initial_tangent(self, x, name, mu):
        self.interface.set_parameter(name, mu + self.delta)
        dflval = self._rhs(x)
        self.interface.set_parameter(name, mu)
        fval = self._rhs(x)
        dflval = (dflval - fval) / self.delta
        jac = self._jac(x)
        dx = self._solve(jac, -dflval)
        dmu = 1
        nrm = math.sqrt(self.zeta * dx.dot(dx) + dmu ** 2)
        dmu /= nrm
        dx /= nrm
        return dx, dmu

    def _return(self, x, mu, dx, dmu, ds, callback, return_step):
        if callback is not None:
            callback(self.interface, x, mu)
        if return_step:
            return x, mu, dx * ds, dmu * ds
        return x, mu

    # -- main loop (Continuation.py:361-482) ----------------------------------
    def continuation(self, x0, parameter_name, start, target, ds, ds_min=0.01, ds_max=1000,
                     dx=None, dmu=None, maxit=1000, detect_bifurcations=False,
                     switch_branches=False, return_step=False, callback=None):
        if detect_bifurcations or switch_branches:
            raise NotImplementedError('bifurcation detection needs an eigenvalue solver')
        self._t0 = time.perf_counter()
        x = x0
        mu = start
        self.zeta = 1 / x.size
        if dx is None or dmu is None:
            dx, dmu = self._initial_tangent(x, parameter_name, mu)
        else:
            dx /= ds
            dmu /= ds
        for j in range(maxit):
            mu0 = mu
            if callback is not None:
                callback(self.interface, x, mu)
            x, mu, dx, dmu, ds = self._step(parameter_name, x, mu, dx, dmu, ds, ds_min, ds_max,
                                            use_predictor=True)
            if (mu >= target and mu0 < target) or (mu <= target and mu0 > target):
                x, mu = self._converge(parameter_name, x, mu, dx, dmu, target,
                                       ds, ds_min, ds_max, maxit - j)
                return self._return(x, mu, dx, dmu, ds, callback, return_step)
            ds = self._adjust_step_size(ds, ds_min, ds_max)
        return self._return(x, mu, dx, dmu, ds, callback, return_step)


class TimeIntegration:
    """Theta-method time integration (TimeIntegration.py:29-115)."""

    def __init__(self, interface, theta=1.0, newton_tolerance=1e-10,
                 maximum_newton_iterations=10, residual_check='F', verbose=False):
        self.interface = interface
        self.verbose = verbose
        self.theta = theta
        self.maximum_newton_iterations = maximum_newton_iterations
        self.newton_tolerance = newton_tolerance
        self.residual_check = residual_check

    def _newton(self, x0, dt):
        x = x0
        b0 = self.interface.rhs(x0)
        mass = self.interface.mass_matrix()
        for k in range(self.maximum_newton_iterations):
            fval = mass @ (x0 - x) + dt * self.theta * self.interface.rhs(x) + dt * (1 - self.theta) * b0
            fval /= self.theta * dt
            if self.residual_check == 'F' or self.verbose:
                fnorm = norm(fval)
            if self.residual_check == 'F' and fnorm < self.newton_tolerance:
                print('Newton converged i %d iterations with ||F||=%e' % (k, fnorm), flush=True)
                break
            jac = self.interface.jacobian(x) - mass / (self.theta * dt)
            dx = self.interface.solve(jac, -fval)
            x = x + dx
            if self.residual_check != 'F' or self.verbose:
                dxnorm = norm(dx)
            if self.residual_check != 'F' and dxnorm < self.newton_tolerance:
                print('Newton converged in %d iterations with ||dx||=%e' % (k, dxnorm), flush=True)
                break
            if self.verbose:
                print('Newton status at iteration %d: ||F||=%e, ||dx||=%e' % (k, fnorm, dxnorm), flush=True)
        return x

    def integration(self, x0, dt, tmax, callback=None):
        x = x0
        t = 0
        if callback:
            callback(self.interface, x, t)
        while t < tmax:
            x = self._newton(x, dt)
            t += dt
            print("t = %f" % t, flush=True)
            if callback:
                callback(self.interface, x, t)
        return x, t
