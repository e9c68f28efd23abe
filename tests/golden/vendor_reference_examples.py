"""Copy the reference's example circuits and networks used as golden inputs.

The reference checkout ships a few small data files under ``examples/``:
OPENQASM circuits (QFT on 2, 3, 5 and 10 qubits, GHZ on 3) and a GHZ-3
network in the reference's JSON form together with an edge plan and the
network the reference produced by contracting along it.  The tests read the
copies in ``tests/golden/reference_examples/`` so that they run where the
checkout is absent.  Run this script from the repository root, with the
reference checkout at ``/root/reference``, to refresh them.
"""
import shutil
import sys
from pathlib import Path

SRC = Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/examples")
DST = Path(__file__).resolve().parent / "reference_examples"
FILES = ["qft_2.qasm", "qft_3.qasm", "qft_5.qasm", "qft_10.qasm", "ghz_3.qasm", "ghz_3.json", "ghz_3_plan.json",
         "ghz_3_contracted.json"]

if __name__ == "__main__":
    DST.mkdir(exist_ok=True)
    for f in FILES:
        shutil.copyfile(SRC / f, DST / f)
        print(f"{f}: {(DST / f).stat().st_size} bytes")
