"""The oracle against the reference's own FCIQMC outputs (the small cases of
tests/golden/reference_fciqmc_runs.json, which the oracle finishes in seconds):
reblocked shift and projected energy within 3 combined standard errors of
HANDE's own run of the same calculation."""

import pytest

from oracle.pyoracle import Oracle
from tests.test_gpu_reference_runs import BY_NAME, run_and_compare


@pytest.mark.parametrize("name", ["hubbard_k_2x2_2e", "H2-sto-3g-replica"])
def test_oracle_matches_reference_run(name):
    run_and_compare(BY_NAME[name], Oracle)
