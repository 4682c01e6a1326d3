"""Seed generators against the reference's own outputs
(tests/golden/seeding.npz from make_golden.py phase seeding: the NumPy
branch of tracking/seeding.py:140-247): the same float32 arrays bit for bit
for every bounds form, and the same refusals."""
import json
from pathlib import Path

import numpy as np
import pytest

from jaxtrace_gb300.seeding import random_seeds, uniform_grid_seeds

GOLDEN = Path(__file__).resolve().parent / "golden" / "seeding.npz"

CALLS = {"rand": lambda b: random_seeds(1000, b, rng_seed=7),
         "rand0": lambda b: random_seeds(0, b),
         "grid": lambda b: uniform_grid_seeds((5, 4, 3), b, True),
         "grid_int": lambda b: uniform_grid_seeds(4, b, False),
         "grid2": lambda b: uniform_grid_seeds((6, 5), b, True),
         "grid2_int": lambda b: uniform_grid_seeds((6, 5), b, False)}


def test_seeds_match_the_reference_bit_for_bit():
    z = np.load(GOLDEN)
    forms = json.loads(str(z["forms"]))
    errors = json.loads(str(z["errors"]))
    checked = refused = 0
    for fname, b in forms.items():
        for cname, fn in CALLS.items():
            key = f"{cname}_{fname}"
            if key in errors:
                with pytest.raises(ValueError) as exc:
                    fn(b)
                assert errors[key]["type"] == "ValueError"
                assert str(exc.value) == errors[key]["message"]
                refused += 1
            else:
                got = fn(b)
                assert got.dtype == np.float32 and got.shape == z[key].shape
                assert np.array_equal(got.view(np.uint32), z[key].astype(np.float32).view(np.uint32)), key
                checked += 1
    assert checked == 21 and refused == 15
