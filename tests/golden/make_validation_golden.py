"""Copies the reference's archived validation results into a small fixture.

Reads, from the reference checkout (the path given as the first argument, else
the one oracle.reference_src() finds: $PIC_REFERENCE_SRC or the oracle build
recipe's), the CSVs its validation driver writes
(src/main_validation.cpp, src/pic/validation.cpp:474-505):
    data/benchmarks/noise_vs_grid.csv, validation.csv, conservation_study.csv,
    two_stream_validation.csv
and writes tests/golden/validation_reference.json. The GPU tests compare the
ported drivers (pic-deposition_gb300/host/pic_validation.cpp) against it.
"""
import csv
import json
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "oracle"))
import oracle  # noqa: E402  (test infrastructure: locates the reference checkout)

src = sys.argv[1] if len(sys.argv) > 1 else oracle.reference_src()
if not src:
    sys.exit("the reference checkout is absent: pass its path or set PIC_REFERENCE_SRC")
bench = os.path.join(src, "data", "benchmarks")
out = {}
for name in ("noise_vs_grid", "validation", "conservation_study", "two_stream_validation"):
    with open(os.path.join(bench, name + ".csv")) as f:
        out[name] = list(csv.DictReader(f))
dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "validation_reference.json")
with open(dst, "w") as f:
    json.dump(out, f, indent=1)
print("wrote", dst)
