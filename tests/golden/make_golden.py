"""Extract the reference's golden vectors for the MSM path into vectors.json.

Run where the helioselene sources are checked out, naming their root in
HELIOSELENE_REF (or passing the fixture's path):

    HELIOSELENE_REF=<helioselene checkout> python tests/golden/make_golden.py

The source file is the reference's own fixture (generated by its
tools/gen_test_vectors.cpp:1107-1159 and checked by src/tests.cpp:6036-6142).
Only the entries that pin this path are kept: point encodings, group law
(add/dbl/negate/scalar_mul), MSM, Pedersen, SSWU map-to-curve, and batch
inversion.  The output is committed so that the test suite never needs the
reference tree at run time.
"""

import json
import os
import sys
from pathlib import Path

KEEP_POINT = ["generator", "identity", "from_bytes", "add", "dbl", "negate",
              "scalar_mul", "msm", "pedersen_commit", "map_to_curve_single",
              "map_to_curve_double"]


def main(src: str) -> None:
    data = json.loads(Path(src).read_text())
    out = {"source": "helioselene test_vectors/helioselene_test_vectors.json",
           "parameters": data["parameters"]}
    for curve in ("helios", "selene"):
        out[curve + "_point"] = {k: data[curve + "_point"][k] for k in KEEP_POINT}
    out["batch_invert"] = data["batch_invert"]
    dst = Path(__file__).with_name("vectors.json")
    dst.write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"wrote {dst} ({dst.stat().st_size} bytes)")


if __name__ == "__main__":
    ref = os.environ.get("HELIOSELENE_REF", "/root/reference")
    main(sys.argv[1] if len(sys.argv) > 1 else str(Path(ref) / "test_vectors" / "helioselene_test_vectors.json"))
