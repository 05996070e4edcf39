"""Freeze the seeded ensembles of the batched configurations.

c3: 64 instances, s uniform in 16..64, seed 0.
c4: 512 instances, s uniform in 8..48, plus 16 instances with s=96, seed 1.
Energy factors log-uniform in [0.5, 2].  Sizes are drawn first, then the
factors, from numpy.random.default_rng(seed) (the package's ``ensemble``).
Usage: python tests/golden/make_ensembles.py
"""
import json
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import __graft_entry__ as ge  # noqa: E402

pkg = ge.load_package()
out = {}
for name, args in {"c3": (0, 64, 16, 64, ()), "c4": (1, 512, 8, 48, (96,) * 16)}.items():
    sizes, factors = pkg.ensemble(*args)
    out[name] = {"seed": args[0], "sizes": sizes.tolist(), "e0_scale": factors.tolist()}
(Path(__file__).resolve().parent / "ensembles.json").write_text(json.dumps(out) + "\n")
print({k: (len(v["sizes"]), sum(s ** 3 for s in v["sizes"])) for k, v in out.items()})
