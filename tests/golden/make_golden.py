"""Generate the golden fixtures under tests/golden/ from the reference checkout.

Run once with REFERENCE set to a checkout of the reference (required; the
script has no default); the outputs are committed, so tests never read the
reference at run time.  Outputs:

  *.bin        byte copies of the reference's small experiment saved states
               (saved_states/TEXPS.bin, Chain_TEXP.bin, PBEXPS.bin,
               Chain_EXP.bin, Strings.bin, MicroStrings.bin) -- FlatBuffers
               `State` tables (new_schema.fbs:86-104) carrying the
               experiment scripts; MicroStrings holds 2048 particles, 4193
               broken bonds and a NaN velocity
  traces.npz   every exported CSV trace of those experiments (data/TEXP_k.csv,
               data/Chain_T_k.csv, data/pb_experiment_k_1.csv, data/Chain_k.csv)
               as float64 arrays [rows, 12] in the column order of
               Settings::save_data (settings.rs:2014-2052):
               Timestamp, X/Y Position, X/Y Velocity, Rotation,
               Rotation Velocity, Data1..Data4, FPS
  TEXP_1_head.csv  the first 12 lines of data/TEXP_1.csv as text: the
               reference's own CSV formatting of those numbers
  Default.bin  byte copy of the Default.bin at the root of the reference
               checkout, a state in neither of its schemas
"""
import glob
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = os.environ.get("REFERENCE")
STATES = ["TEXPS.bin", "Chain_TEXP.bin", "PBEXPS.bin", "Chain_EXP.bin", "Strings.bin", "MicroStrings.bin"]
TRACE_GLOBS = ["TEXP_*.csv", "Chain_T_*.csv", "pb_experiment_*_1.csv", "Chain_[0-9]*.csv"]


def main():
    if not REFERENCE:
        sys.exit("set REFERENCE to the reference checkout")
    src_states = os.path.join(REFERENCE, "saved_states")
    src_data = os.path.join(REFERENCE, "data")
    if not os.path.isdir(src_states):
        sys.exit("reference checkout not found at %s" % REFERENCE)
    for name in STATES:
        shutil.copyfile(os.path.join(src_states, name), os.path.join(HERE, name))
    traces = {}
    for pat in TRACE_GLOBS:
        for path in sorted(glob.glob(os.path.join(src_data, pat))):
            key = os.path.splitext(os.path.basename(path))[0]
            rows = np.loadtxt(path, delimiter=",", skiprows=1, dtype=np.float64, ndmin=2)
            traces[key] = rows
    np.savez_compressed(os.path.join(HERE, "traces.npz"), **traces)
    shutil.copyfile(os.path.join(REFERENCE, "Default.bin"), os.path.join(HERE, "Default.bin"))
    with open(os.path.join(src_data, "TEXP_1.csv")) as f:
        head = [next(f) for _ in range(12)]
    with open(os.path.join(HERE, "TEXP_1_head.csv"), "w") as f:
        f.writelines(head)
    print("wrote %d states, %d traces" % (len(STATES), len(traces)))


if __name__ == "__main__":
    main()
