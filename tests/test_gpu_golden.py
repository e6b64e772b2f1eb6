"""The CUDA engine against the committed golden fixtures (clODE's own kernels
compiled as C) and the known answers of the reference's test suite.
Fixtures marked exact are compared bit for bit; the others with the
fixture's tolerance (they call exp/pow/log)."""
import pytest

from tests import known_answers as KA
from tests.golden.scenarios import scenarios
from tests.parity import run_engine
from tests.test_oracle import compare_to_fixture

pytestmark = pytest.mark.gpu
SCEN = scenarios()


@pytest.mark.parametrize("schedule", [0, 1])
@pytest.mark.parametrize("name", sorted(SCEN))
def test_engine_matches_golden_fixture(name, schedule):
    sc, exact, rtol = SCEN[name]
    compare_to_fixture(run_engine(sc, options={"schedule": schedule}), name)


@pytest.mark.parametrize("check", KA.ALL, ids=lambda f: f.__name__)
def test_engine_known_answers(check):
    check(run_engine)
