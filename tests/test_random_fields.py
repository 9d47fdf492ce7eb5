"""The product's random-field generator (rewl_generate_fields, host only) against the
reference's own Disorder::generate_random_field run from the same seeds by the reference
harness (tests/golden/random_fields.json, written by tests/golden/make_golden.py fields):
bit-identical doubles."""
import json

import numpy as np
import pytest

from conftest import GOLDEN


def test_fields_match_the_reference_generator(engine_lib):
    rg = engine_lib
    for case in json.loads((GOLDEN / "random_fields.json").read_text()):
        ref = np.array([float.fromhex(x) for x in case["fields"]])
        got = rg.generate_fields(case["seed"], case["strength"], len(ref), case["distribution"])
        assert np.array_equal(got.view(np.uint64), ref.view(np.uint64)), case["seed"]


def test_fields_statistics_and_arguments(engine_lib):
    rg = engine_lib
    h = rg.generate_fields(11, 0.5, 20000)
    assert abs(h.mean()) < 0.02 and abs(h.std() - 0.5) < 0.02
    u = rg.generate_fields(11, 0.5, 20000, rg.DISORDER_UNIFORM)
    assert u.min() >= -1.0 and u.max() <= 1.0 and abs(u.std() - 2.0 / np.sqrt(3.0) * 0.5) < 0.02
    assert rg.generate_fields(3, 1.0, 0).shape == (0,)
    with pytest.raises(rg.REWLError):
        rg.generate_fields(3, 1.0, 10, 7)
