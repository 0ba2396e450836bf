"""The ctypes mirrors of the C ABI's structs (helio_gb300/native.py) against the header
itself: a small C program built with the host compiler prints every struct's size and
field offsets, which must equal the ctypes layout (a mismatch would pass garbage across
the boundary without any error)."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

from helio_gb300 import layouts as L
from helio_gb300 import native as N

ROOT = Path(__file__).resolve().parent.parent

# (C struct, ctypes class)
PAIRS = [
    ("hl_froxel_params", N.FroxelParams), ("hl_froxel_lists", N.FroxelLists), ("hl_gbuffer", N.GBuffer),
    ("hl_light_grid", N.LightGrid), ("hl_target", N.Target), ("hl_view", N.View),
    ("hl_batch_config", N.BatchConfig), ("hl_fragment_params", N.FragmentParams), ("hl_texture", N.Texture),
    ("hl_shadow_maps", N.ShadowMaps), ("hl_rc_cascade", N.RcCascade), ("hl_shade_bindings", N.ShadeBindings),
    ("hl_reflection_inputs", N.ReflectionInputs), ("hl_gbuffer_targets", N.GBufferTargets),
    ("hl_reflection_env", N.ReflectionEnv),
]
# (C struct, numpy record dtype) for the records the oracle and the tests build
DTYPES = [
    ("hl_froxel_params", L.FROXEL_PARAMS), ("hl_fragment", L.FRAGMENT), ("hl_surface", L.SURFACE),
    ("hl_texture", L.TEXTURE), ("hl_shadow_maps", L.SHADOW_MAPS), ("hl_rc_cascade", L.RC_CASCADE),
    ("hl_reflection_env", L.REFLECTION_ENV),
]


def _c_fields(cname):
    names = [f[0] for c, cls in PAIRS if c == cname for f in cls._fields_]
    names += [n for c, dt in DTYPES if c == cname for n in dt.names if not n.startswith("_")]
    return sorted(set(names))


@pytest.fixture(scope="module")
def c_layouts(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "helio_gb300.h"', "int main(void) {"]
    for cname in sorted({c for c, _ in PAIRS} | {c for c, _ in DTYPES}):
        lines.append(f'printf("{cname} @sizeof %zu\\n", sizeof({cname}));')
        for f in _c_fields(cname):
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    d = tmp_path_factory.mktemp("structs")
    src, exe = d / "structs.c", d / "structs"
    src.write_text("\n".join(lines) + "\n")
    r = subprocess.run([cc, "-std=c11", "-Wall", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    table = {}
    for line in out.splitlines():
        s, k, v = line.split()
        table[(s, k)] = int(v)
    return table


@pytest.mark.parametrize("cname,cls", PAIRS, ids=[p[0] for p in PAIRS])
def test_ctypes_layout_matches_header(c_layouts, cname, cls):
    assert C.sizeof(cls) == c_layouts[(cname, "@sizeof")], cname
    for f in cls._fields_:
        assert getattr(cls, f[0]).offset == c_layouts[(cname, f[0])], (cname, f[0])


@pytest.mark.parametrize("cname,dt", DTYPES, ids=[p[0] for p in DTYPES])
def test_numpy_records_match_header(c_layouts, cname, dt):
    assert dt.itemsize == c_layouts[(cname, "@sizeof")], cname
    for n in dt.names:
        if not n.startswith("_"):
            assert dt.fields[n][1] == c_layouts[(cname, n)], (cname, n)
