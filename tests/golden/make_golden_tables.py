"""Regenerate tests/golden/ref_tables.json from the reference's own host code.

Builds oracle/_ref/ref_dump (oracle/Makefile.ref compiles PhantomFHE's src/host/*.cu
unmodified, from the reference checkout named by REF) and stores its output.  Arrays
longer than 64 words are stored as the SHA-256 of their little-endian uint64 bytes plus
their first and last 4 entries; shorter arrays are stored in full.  Run from the repo
root:  python tests/golden/make_golden_tables.py [REF]  (default: $PHANTOM_FHE_REFERENCE)
"""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def compact(obj):
    if isinstance(obj, dict):
        return {k: compact(v) for k, v in obj.items()}
    if isinstance(obj, list) and obj and isinstance(obj[0], int) and len(obj) > 64:
        a = np.array(obj, dtype=np.uint64)
        return {"len": len(obj), "sha256": hashlib.sha256(a.tobytes()).hexdigest(),
                "head": obj[:4], "tail": obj[-4:]}
    if isinstance(obj, list):
        return [compact(v) for v in obj]
    return obj


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PHANTOM_FHE_REFERENCE")
    if not ref:
        sys.exit("name the PhantomFHE source checkout: make_golden_tables.py REF or PHANTOM_FHE_REFERENCE=REF")
    subprocess.check_call(["make", "-s", "-f", "oracle/Makefile.ref", f"REF={ref}", "-j8"], cwd=ROOT)
    raw = subprocess.check_output([os.path.join(ROOT, "oracle", "_ref", "ref_dump")])
    data = compact(json.loads(raw))
    out = os.path.join(ROOT, "tests", "golden", "ref_tables.json")
    with open(out, "w") as f:
        json.dump(data, f, separators=(",", ":"))
    print(out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
