"""The full-size slab fixture (tests/golden/slab_c3) keeps no input files,
only the seeded generator's arguments and the SHA-256 of what it writes: the
generator must write the same bytes here as where the fixture was made."""
import json
import os
import sys

from conftest import GOLDEN


def test_c3_generator_reproduces_the_fixture_inputs(tmp_path):
    sys.path.insert(0, GOLDEN)
    import make_c3_golden as g
    meta = json.load(open(os.path.join(GOLDEN, "slab_c3", "meta.json")))
    assert meta["spec"] == g.SPEC
    g.spec().write(str(tmp_path))
    assert g.file_hashes(str(tmp_path)) == meta["sha256"]
