"""The full-size slab fixture (tests/golden/slab_c3) keeps no input files,
only the seeded generator's arguments and the SHA-256 of what it writes: the
generator must write the same bytes here as where the fixture was made.  The
oracle's field (a direct DFT) is checked against the reference's kiss_fft
samples on the first 200 positions."""
import json
import os
import sys

import numpy as np

import oracle
from conftest import GOLDEN
from mechafm_gb300.scan import Input


def test_c3_generator_reproduces_the_fixture_inputs(tmp_path):
    sys.path.insert(0, GOLDEN)
    import make_c3_golden as g
    meta = json.load(open(os.path.join(GOLDEN, "slab_c3", "meta.json")))
    assert meta["spec"] == g.SPEC
    g.spec().write(str(tmp_path))
    assert g.file_hashes(str(tmp_path)) == meta["sha256"]
    g.field_spec().write(str(tmp_path / "field"))
    assert g.file_hashes(str(tmp_path / "field")) == meta["sha256_field"]


def test_c3_field_samples_match_the_oracle(tmp_path):
    sys.path.insert(0, GOLDEN)
    import make_c3_golden as g
    ref = np.load(os.path.join(GOLDEN, "slab_c3", "ref.npz"))
    want = ref["es_fe"][:200]
    assert np.abs(want).max() > 0.1
    desc = Input(g.field_spec().write(str(tmp_path))).desc()
    got = oracle.sample(desc, ref["es_pts"][:200], what=1)
    err = np.abs(got - want) / np.maximum(np.abs(want), 1e-2)
    assert err.max() <= 1e-9, err.max()
