"""The Rust RenderPass shim (rust/helio-pass-gb300) against the C ABI it binds, CPU only.
Rust cannot be compiled in this image, so the check is structural: every entry point
include/helio_gb300.h declares is declared in the shim's extern block with the same
number of parameters, nothing else is, and the repr(C) structs list the header's
fields in the header's order; the passes keep the reference's pass names and
resource names (light-cull/src/lib.rs:194-206, deferred-light/src/lib.rs:790-830)."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "helio_gb300.h"
SYS = ROOT / "rust" / "helio-pass-gb300" / "src" / "sys.rs"
LIB = ROOT / "rust" / "helio-pass-gb300" / "src" / "lib.rs"


def _strip_c_comments(text):
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def _arity(params: str) -> int:
    params = " ".join(params.split())
    if params in ("", "void"):
        return 0
    return params.count(",") + 1


def header_functions():
    text = _strip_c_comments(HEADER.read_text())
    out = {}
    for m in re.finditer(r"^(?:hl_status|uint32_t|const char\*)\s+(hl_\w+)\s*\(([^;]*?)\)\s*;", text, flags=re.M | re.S):
        out[m.group(1)] = _arity(m.group(2))
    return out


def rust_functions():
    text = SYS.read_text()
    block = text[text.index('extern "C" {'):]
    out = {}
    for m in re.finditer(r"pub fn (hl_\w+)\s*\(([^)]*)\)", block, flags=re.S):
        args = m.group(2).strip().rstrip(",")
        out[m.group(1)] = 0 if not args else args.count(",") + 1
    return out


def header_struct_fields(name):
    text = _strip_c_comments(HEADER.read_text())
    m = re.search(r"typedef struct %s \{(.*?)\}\s*%s;" % (name, name), text, flags=re.S)
    fields = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        decl = re.sub(r"\[[^\]]*\]", "", decl)
        names = decl.split()[-1] if "," not in decl else decl
        # "uint32_t grid_x, grid_y, grid_z" -> three fields
        parts = [p.strip() for p in decl.split(",")]
        first = parts[0].split()[-1].lstrip("*")
        fields.append(first)
        fields.extend(p.lstrip("*") for p in parts[1:])
    return fields


def rust_struct_fields(name):
    text = SYS.read_text()
    m = re.search(r"pub struct %s \{(.*?)\n\}" % name, text, flags=re.S)
    return re.findall(r"pub (\w+):", m.group(1))


def test_every_entry_point_is_bound_with_its_arity():
    h, r = header_functions(), rust_functions()
    assert len(h) >= 25
    assert set(h) == set(r), (sorted(set(h) - set(r)), sorted(set(r) - set(h)))
    bad = {k: (h[k], r[k]) for k in h if h[k] != r[k]}
    assert not bad, bad


def test_repr_c_structs_list_the_header_fields_in_order():
    for name in ["hl_froxel_params", "hl_froxel_lists", "hl_gbuffer", "hl_light_grid", "hl_target", "hl_shadow_maps",
                 "hl_rc_cascade", "hl_shade_bindings", "hl_reflection_inputs", "hl_reflection_env", "hl_fragment_params", "hl_surface",
                 "hl_texture", "hl_gbuffer_targets", "hl_view", "hl_batch_config"]:
        assert rust_struct_fields(name) == header_struct_fields(name), name


def test_passes_keep_the_reference_names():
    lib = LIB.read_text()
    assert '"LightCull"' in lib and '"DeferredLight"' in lib
    assert '&["tile_light_lists", "tile_light_counts"]' in lib
    assert '&["pre_aa"]' in lib
    for name in ["gbuffer", "depth", "tile_light_lists", "tile_light_counts", "pre_aa", "ssao", "rc_view"]:
        assert f'"{name}"' in lib
    # DeferredGlobals: the 112-byte uniform, field for field
    fields = re.search(r"pub struct DeferredGlobals \{(.*?)\n\}", lib, flags=re.S).group(1)
    assert re.findall(r"pub (\w+):", fields) == [
        "frame", "delta_time", "light_count", "ambient_intensity", "ambient_color", "rc_world_min", "rc_world_max",
        "csm_splits", "debug_mode", "has_rc_gi", "num_tiles_x", "reflection_capture_count", "enable_reflections",
        "enable_env_reflections", "_pad"]
    assert "InvalidPassConfig" in lib and "cull_cache_key" in lib
