"""Saved-state access for the tests: the package's FlatBuffers reader and
writer (physics-sim_gb300/state_io.py), under the names the tests use."""
from state_io import (decode_settings, grid_capacity, load_state, parse, save_state,  # noqa: F401
                      uniform_from)
