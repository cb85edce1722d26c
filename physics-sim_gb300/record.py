"""Recording and CSV export of the reference's experiment data.

The reference's `Advance` with `Record` on (src/client.rs:931-974) steps one
at a time and, after each step, reads the whole state back and appends the
datum of the selected particles (State::get_datum, src/state.rs:708-737)
with the timestamp dT * generation (an f32 product, stored as f64) and the
frame rate; `Settings::save_data` (src/settings.rs:2014-2052) writes those
rows as CSV.  Here the datum of every step is gathered on the device
(dem_record) and read back once per call; `write_csv` writes the same
header and the numbers as the reference prints them (Rust's `{}` for f64:
the shortest digits that read back to the same value, never an exponent).
"""
from decimal import ROUND_HALF_UP, Decimal

import numpy as np

HEADER = ("Timestamp,X Position,Y Position,X Velocity,Y Velocity,Rotation,Rotation Velocity,"
          "Data1,Data2,Data3,Data4,FPS")


def advance_recording(ctx, ticks, selections, dt, generation):
    """client.rs:948-956: `ticks` recorded steps, then the one unrecorded step
    the reference's loop runs after them.  Returns (rows [ticks, 11] with the
    timestamp first, or None when nothing is selected; the generation
    counter after the recorded steps)."""
    data = ctx.record(ticks, selections)
    ctx.step(1)
    if data is None:
        return None, generation + ticks
    gen = generation + 1 + np.arange(ticks)
    t = (np.float32(dt) * gen.astype(np.float32)).astype(np.float32).astype(np.float64)
    return np.column_stack([t, data]), generation + ticks


def format_f64(x):
    """Rust's Display of an f64: the fewest significant digits that read back
    to the same value, positional.  When the value lies exactly halfway
    between the two candidates of that length, Rust prints the one of larger
    magnitude (Python's shortest repr prints the even one)."""
    x = float(x)
    if x != x:
        return "NaN"
    if x in (float("inf"), float("-inf")):
        return "inf" if x > 0 else "-inf"
    s = np.format_float_positional(x, unique=True, trim="-")
    if x == 0.0:
        return s
    q = Decimal(s)
    digits = len(s.replace("-", "").replace(".", "").lstrip("0"))
    unit = Decimal(1).scaleb(q.adjusted() - digits + 1)
    up = Decimal(x).quantize(unit, rounding=ROUND_HALF_UP)
    if up != q and float(up) == x:
        return format(up, "f")
    return s


def write_csv(path, rows, fps=None):
    """Settings::save_data: rows [k, 11] (timestamp and the ten datum
    columns) plus an FPS column (`fps`: one value per row, a scalar, or None
    for 0), with the reference's header."""
    rows = np.asarray(rows, np.float64).reshape(-1, 11)
    f = np.zeros(rows.shape[0]) if fps is None else np.broadcast_to(np.asarray(fps, np.float64), rows.shape[0])
    with open(path, "w") as out:
        out.write(HEADER + "\n")
        for r, v in zip(rows, f):
            out.write(",".join(format_f64(x) for x in list(r) + [v]) + "\n")
