"""The C restatement (oracle/fs_oracle.c) against the fixtures recorded from
the reference's own code (tests/golden/make_golden.py): bit-exact on every
observable array, for every step method, an obstacle and a fluid source."""
import os

import numpy as np
import pytest

from tests.golden import make_golden as mg


@pytest.mark.parametrize("case", sorted(mg.CASES))
def test_restatement_matches_reference_fixture(case, golden_dir):
    ref = np.load(os.path.join(golden_dir, case + ".npz"))
    got = mg.run_case("restatement", case)
    assert sorted(got) == sorted(ref.files)
    for key in ref.files:
        a, b = got[key], ref[key]
        assert a.shape == b.shape, key
        if key.endswith("_cg"):
            assert a[0] == b[0] and a[2] == b[2], key
            assert a[1] == b[1], key
        else:
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), key
