"""The Simulation kernels of a batch whose scenes share their settings read
those settings from the launch (PS_SHARED) and everything else from the
scene's record.  A field read through the shared record must be one that
shared_settings (csrc/dem_world.cuh) copies, or every scene would read 0
there.  This checks the kernels' source against that function: the fields
interact_particle and lom_core read through `U`, and every field
linear_model reads (it is handed `U`)."""
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "physics-sim_gb300", "csrc")


def _body(src, signature):
    """Text of the function whose definition starts with `signature`."""
    at = src.index(signature)
    open_at = src.index("{", at)
    depth = 0
    for k in range(open_at, len(src)):
        if src[k] == "{":
            depth += 1
        elif src[k] == "}":
            depth -= 1
            if depth == 0:
                return src[open_at:k + 1]
    raise AssertionError("unbalanced braces after " + signature)


def _copied_fields():
    hdr = open(os.path.join(CSRC, "dem_world.cuh")).read()
    body = _body(hdr, "inline ScenePar shared_settings(")
    return set(re.findall(r"\bk\.((?:p\.)?[a-zA-Z_0-9]+)\s*=", body))


def test_fields_read_through_the_shared_record_are_copied():
    src = open(os.path.join(CSRC, "dem_kernels.cu")).read()
    read = set()
    for sig in ("__device__ __forceinline__ void interact_particle(",
                "__device__ __forceinline__ void lom_core("):
        read |= set(re.findall(r"\bU\.((?:p\.)?[a-zA-Z_0-9]+)", _body(src, sig)))
    read |= set(re.findall(r"\bP\.((?:p\.)?[a-zA-Z_0-9]+)",
                           _body(src, "__device__ __forceinline__ F3 linear_model(")))
    copied = _copied_fields()
    assert read, "no shared-record reads found: the source layout changed"
    assert read <= copied, "read through the shared record but not copied: %s" % sorted(read - copied)


def test_linear_model_is_handed_the_shared_record():
    src = open(os.path.join(CSRC, "dem_kernels.cu")).read()
    calls = re.findall(r"linear_model<[^>]*>\((\w+),", _body(src, "__device__ __forceinline__ void interact_particle("))
    assert calls and set(calls) == {"U"}
