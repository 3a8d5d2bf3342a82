"""Many independent instances solved concurrently, each on its own stream
(the batched configuration), against the same instances solved alone and
against the oracle's residual."""

import numpy as np
import pytest

from oracle.solve import Interface as OracleInterface

SPECS = [{'nx': 16, 'target': 300.0, 'ds': 100.0, 'tolerance': 1e-10},
         {'nx': 24, 'target': 800.0, 'ds': 100.0, 'tolerance': 1e-10},
         {'nx': 20, 'ny': 12, 'target': 1500.0, 'ds': 150.0, 'tolerance': 1e-10},
         {'nx': 16, 'target': 0.0, 'tolerance': 1e-10}]


@pytest.mark.gpu
def test_solve_many_matches_instances_solved_alone(built_lib):
    from transiflow_gb300.batch import solve_instance, solve_many
    many = solve_many(SPECS)
    for spec, res in zip(SPECS, many):
        alone = solve_instance(spec)
        assert abs(res['mu'] - spec['target']) < 1e-3
        assert res['fnorm'] <= 1e-10
        scale = max(1.0, np.abs(alone['x']).max())
        np.testing.assert_allclose(res['x'], alone['x'], rtol=0, atol=1e-9 * scale)


@pytest.mark.gpu
def test_solve_many_states_are_roots_of_the_oracle(built_lib):
    from transiflow_gb300.batch import solve_many
    for spec, res in zip(SPECS, solve_many(SPECS, concurrency=2)):
        ny = spec.get('ny', spec['nx'])
        o = OracleInterface({'Reynolds Number': res['mu']}, spec['nx'], ny)
        assert np.linalg.norm(o.rhs(res['x'])) <= 1e-9
