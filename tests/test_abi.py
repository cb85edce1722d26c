"""CPU tests of the C ABI library: it loads, exports every declared entry point,
its structs have the reference's layouts, and its host-only helpers agree
with the reference's formulas.  No compute call needs a GPU here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import dem
import dem_scenes
import state_io
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


@pytest.fixture(scope="module")
def L():
    import build_lib
    build_lib.build()
    return dem.lib()


def _declared():
    names = set()
    for f in os.listdir(INCLUDE):
        if not f.endswith(".h"):
            continue
        txt = open(os.path.join(INCLUDE, f)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(dem_\w+)\s*\(", txt, flags=re.M):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported(L):
    declared = _declared()
    assert "dem_step" in declared and "dem_create" in declared
    for name in sorted(declared):
        assert hasattr(L, name), "libdemgb.so does not export %s" % name
    assert set(dem.SYMBOLS) <= declared


def test_abi_version(L):
    assert L.dem_abi_version() == 1


def test_struct_layouts(L):
    # the settings uniform is 29 four-byte words, like collision_settings()
    assert C.sizeof(dem.Params) == 29 * 4
    assert C.sizeof(dem.GridInfo) == 16
    assert C.sizeof(dem.BreakEvent) == 24
    assert dem.Params.dT.offset == 19 * 4
    assert dem.Params.particles.offset == 28 * 4
    e = dem.Ext()
    L.dem_ext_defaults(C.byref(e))
    assert e.bond_lambda == pytest.approx(0.5) and e.diagnostics == 1 and e.use_f64 == 0


@pytest.mark.parametrize("fixture", ["TEXPS.bin", "Chain_TEXP.bin", "PBEXPS.bin", "Strings.bin"])
def test_grid_capacity_matches_reference_formula(L, golden_dir, fixture):
    raw = state_io.parse(open(os.path.join(golden_dir, fixture), "rb").read())
    scene, uni, info = state_io.load_state(os.path.join(golden_dir, fixture))
    got = dem.grid_capacity(uni, raw["radii"], info["particles"])
    assert got[0] == pytest.approx(scene["grid"][0], rel=0, abs=0)
    assert got[1:] == tuple(scene["grid"][1:])
    rad = raw["radii"]
    o = oracle.grid_capacity(uni["hor_bound"], uni["vert_bound"], float(rad.max()), float(rad.min()),
                             rad.min() != rad.max(), info["particles"])
    assert got == o


def test_chain_builder_equals_regen_bonds():
    sc, _, _ = dem_scenes.c1_chains(chains=4, length=9)
    b, c = oracle.regen_bonds(sc["pos"], sc["radii"])
    assert np.array_equal(b, sc["bonds"])
    assert np.array_equal(c, sc["contacts"])


def test_create_without_gpu_reports_error(L):
    """On a machine without a GPU the product path fails loudly, never silently."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    sc, p, ext = dem_scenes.c0_settle(n=64, box=(32, 32), spacing=2.6)
    with pytest.raises(dem.DemError) as ei:
        dem.Context(sc, p)
    assert ei.value.code in (-3, -1)


def test_invalid_scene_is_rejected_before_device_work(L):
    sc, p, _ = dem_scenes.c0_settle(n=16, box=(32, 32), spacing=2.6)
    sc["material_pointers"][3] = 7   # beyond the single material
    st = dem.make_scene(sc)
    pp = dem.make_params(p)
    e = dem.make_ext()
    h = C.c_void_p()
    rc = L.dem_create(C.byref(st), C.byref(pp), C.byref(e), -1, C.byref(h))
    assert rc != 0 and not h.value
    assert L.dem_last_error(None)


_C_STRUCTS = [("Params", "dem_params"), ("GridInfo", "dem_grid_info"), ("Ext", "dem_ext"),
              ("Scene", "dem_scene"), ("BreakEvent", "dem_break_event"), ("Stats", "dem_stats"),
              ("ServerConfig", "dem_server_config"), ("ServerStats", "dem_server_stats"),
              ("TuneResult", "dem_tune_result")]


def test_headers_compile_as_c_and_match_the_binding(tmp_path):
    """dem.h and dem_debug.h compile as C11 with warnings as errors, and every
    struct's size and field offsets, as a C compiler lays them out, equal the
    binding's ctypes mirrors (the layouts a Rust or C host of the reference
    binds against)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "dem.h"', '#include "dem_debug.h"',
             "int main(void) {"]
    for py, c in _C_STRUCTS:
        lines.append('    printf("%s sizeof %%zu\\n", sizeof(%s));' % (py, c))
        for f in getattr(dem, py)._fields_:
            lines.append('    printf("%s %s %%zu\\n", offsetof(%s, %s));' % (py, f[0], c, f[0]))
    lines += ["    return 0;", "}"]
    src = tmp_path / "layouts.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layouts"
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", INCLUDE, str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for line in out:
        if line:
            py, field, val = line.split()
            got[(py, field)] = int(val)
    for py, _ in _C_STRUCTS:
        cls = getattr(dem, py)
        assert got[(py, "sizeof")] == C.sizeof(cls), py
        for f in cls._fields_:
            assert got[(py, f[0])] == getattr(cls, f[0]).offset, (py, f[0])
