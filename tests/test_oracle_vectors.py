"""The oracle against its own committed vectors (tests/golden/oracle_vectors.json,
made by tests/golden/make_oracle_vectors.py): the same outputs, bit for bit,
so a change that moved the oracle (and with it the kernels it checks) shows
here.  The digests do not depend on the oracle's thread count."""
import json
import sys
from pathlib import Path

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_oracle_reproduces_its_vectors(orc):
    sys.path.insert(0, str(GOLDEN))
    try:
        import make_oracle_vectors as gen
    finally:
        sys.path.pop(0)
    want = json.loads((GOLDEN / "oracle_vectors.json").read_text())
    got = gen.compute()
    assert sorted(got) == sorted(want)
    changed = [k for k in want if got[k] != want[k]]
    assert not changed, f"oracle outputs changed: {changed}"
