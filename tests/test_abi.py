"""The C-ABI library loads and exports the declared interface (no GPU needed)."""
import ctypes as C
import subprocess

import numpy as np

from underwaterworld_gb300 import abi
from underwaterworld_gb300.chunk import make_descs


def test_library_exports_every_declared_symbol(built_lib):
    declared = abi.declared_functions()
    assert len(declared) >= 20
    L = C.CDLL(str(built_lib))
    for name in declared:
        assert hasattr(L, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(built_lib)], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert exported == set(declared), exported ^ set(declared)
    assert set(abi._SIGS) == set(declared)


def test_abi_version_and_status_strings(built_lib):
    assert abi.lib().uww_abi_version() == 3
    assert abi.status_string(abi.UWW_ERR_CAPACITY) == "output capacity exceeded"


def test_struct_layouts():
    assert C.sizeof(abi.ChunkDesc) == 32
    assert C.sizeof(abi.ChunkRecord) == 32
    assert abi.VERT_COLOR_DTYPE.itemsize == 24  # draw::VertColor stride (draw.rs:19)
    assert C.sizeof(abi.Params) == 4 * (16 + 16 + 6)


def test_reference_params(built_lib):
    p = abi.reference_params()
    assert (p.seed, p.octaves, p.chunk_size) == (0, 3, 16)
    assert p.base_freq == np.float32(1 / 16)
    assert (p.lacunarity, p.persistence, p.amplitude, p.normalize) == (2.0, 0.5, 1.0, 1)
    assert p.bias_mode == abi.UWW_BIAS_TERRACED and (p.bias_a, p.bias_b, p.bias_c) == (16.0, 32.0, 0.25)
    assert p.iso_level == np.float32(-0.1)
    assert (p.color_min_z, p.color_max_z) == (-2.0, 2.0)


def test_python_reference_params_equal_the_librarys(built_lib):
    """layout.reference_params() (what the oracle and the benchmark's reference
    arm use without loading the library) is byte for byte uww_params_reference()."""
    from underwaterworld_gb300 import layout
    assert bytes(layout.reference_params()) == bytes(abi.reference_params())


def test_layout_cells(built_lib):
    d = make_descs(np.zeros((3, 3)), [12, 24, 48])
    raw = np.zeros(3, dtype=abi.CHUNK_DESC_DTYPE)
    raw["cells"] = [12, 24, 48]
    tc, ts = C.c_uint64(), C.c_uint64()
    assert abi.lib().uww_layout_cells(raw.ctypes.data_as(C.c_void_p), 3, C.byref(tc), C.byref(ts)) == 0
    np.testing.assert_array_equal(raw["cell_offset"], d["cell_offset"])
    np.testing.assert_array_equal(raw["sample_offset"], d["sample_offset"])
    assert tc.value == 12**3 + 24**3 + 48**3 and ts.value == 13**3 + 25**3 + 49**3
    raw["cells"][1] = 0
    assert abi.lib().uww_layout_cells(raw.ctypes.data_as(C.c_void_p), 3, None, None) == abi.UWW_ERR_INVALID_ARG


def test_invalid_arguments_are_rejected_on_the_host(built_lib):
    L = abi.lib()
    p = abi.reference_params()
    h = C.c_void_p()
    bad = p.copy()
    bad.octaves = 0
    assert L.uww_ctx_create(C.byref(bad), None, C.byref(h)) == abi.UWW_ERR_INVALID_ARG
    bad = p.copy()
    bad.math_mode = 7
    assert L.uww_ctx_create(C.byref(bad), None, C.byref(h)) == abi.UWW_ERR_INVALID_ARG
    for field, value in (("bias_a", float("inf")), ("bias_c", float("nan")), ("color_max_z", float("inf")),
                         ("outputs", 16)):
        bad = p.copy()
        setattr(bad, field, value)
        assert L.uww_ctx_create(C.byref(bad), None, C.byref(h)) == abi.UWW_ERR_INVALID_ARG, field
    assert L.uww_ctx_create(C.byref(p), None, None) == abi.UWW_ERR_INVALID_ARG
    assert L.uww_build_chunks(None, None, 0, 12, None) == abi.UWW_ERR_INVALID_ARG
    assert L.uww_perm_table(0, None) == abi.UWW_ERR_INVALID_ARG


def test_totals_status_maps_every_error_flag():
    """The Python mirror reads a device build's totals words as the C host path
    does: timeout first, then a bad descriptor or an out-of-range per-cell or
    per-sample write, then a capacity overflow."""
    from underwaterworld_gb300.chunk import totals_status
    t = lambda ovf, flags: np.array([10, 30, ovf, flags], np.uint64)
    assert totals_status(t(0, 0)) == abi.UWW_OK
    assert totals_status(t(3, 0)) == abi.UWW_ERR_CAPACITY
    assert totals_status(t(0, abi.UWW_ERRFLAG_BAD)) == abi.UWW_ERR_INVALID_ARG
    assert totals_status(t(0, abi.UWW_ERRFLAG_RANGE)) == abi.UWW_ERR_INVALID_ARG
    assert totals_status(t(3, abi.UWW_ERRFLAG_RANGE | abi.UWW_ERRFLAG_TIMEOUT)) == abi.UWW_ERR_TIMEOUT


def test_rust_binding_declares_every_entry_point():
    """The Rust `extern "C"` block of the integration guide declares every
    function of include/uww.h, each once."""
    import re
    from pathlib import Path
    text = (Path(__file__).resolve().parent.parent / "INTEGRATION.md").read_text()
    bound = re.findall(r"pub fn (uww_\w+)\(", text)
    assert sorted(bound) == sorted(set(bound))
    assert set(bound) == set(abi.declared_functions()), set(bound) ^ set(abi.declared_functions())


def test_ctypes_mirrors_match_the_header_layouts(tmp_path):
    """Every struct of include/uww.h has the same size and field offsets in the
    Python mirror (compiled with gcc against the header)."""
    import shutil
    from pathlib import Path
    import pytest
    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    mirrors = {"uww_params": abi.Params, "uww_chunk_desc": abi.ChunkDesc, "uww_chunk_record": abi.ChunkRecord,
               "uww_mesh_out": abi.MeshOut, "uww_ray_scene": abi.RayScene,
               "uww_schedule_params": abi.ScheduleParams, "uww_camera_uniform": abi.CameraUniform,
               "uww_tuning": abi.Tuning, "uww_launch_shape": abi.LaunchShape}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "uww.h"', "int main(void) {"]
    for cname, cls in mirrors.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in cls._fields_:
            lines.append(f'printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines.append('printf("uww_vert_color size %zu\\n", sizeof(uww_vert_color));')
    for f in abi.VERT_COLOR_DTYPE.names:
        lines.append(f'printf("uww_vert_color {f} %zu\\n", offsetof(uww_vert_color, {f}));')
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    inc = Path(__file__).resolve().parent.parent / "include"
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", f"-I{inc}", str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        s, f, v = line.split()
        got[(s, f)] = int(v)
    for cname, cls in mirrors.items():
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for f in cls._fields_:
            assert got[(cname, f[0])] == getattr(cls, f[0]).offset, (cname, f[0])
    assert got[("uww_vert_color", "size")] == abi.VERT_COLOR_DTYPE.itemsize
    for f in abi.VERT_COLOR_DTYPE.names:
        assert got[("uww_vert_color", f)] == abi.VERT_COLOR_DTYPE.fields[f][1], f


def test_ctypes_signatures_match_the_header_prototypes():
    """Each function's ctypes signature has the header prototype's argument
    count, integer widths and return kind (int status, pointer, or void)."""
    import re
    text = re.sub(r"/\*.*?\*/", "", abi.HEADER.read_text(), flags=re.S)
    protos = re.findall(r"^\s*((?:const )?\w+\s*\**)\s*(uww_\w+)\s*\(([^;]*)\)\s*;", text, flags=re.M)
    assert {name for _, name, _ in protos} == set(abi.declared_functions())
    widths = {"uint32_t": C.c_uint32, "int32_t": C.c_int32, "uint64_t": C.c_uint64, "int": C.c_int,
              "size_t": C.c_size_t, "float": C.c_float, "double": C.c_double}
    for ret, name, args in protos:
        res, argtypes = abi._SIGS[name]
        params = [] if " ".join(args.split()) in ("", "void") else [a.strip() for a in args.split(",")]
        assert len(params) == len(argtypes), name
        for decl, t in zip(params, argtypes):
            base = decl.replace("const ", "").split()[0]
            if "*" in decl or "[" in decl:
                assert t in (C.c_void_p, C.c_char_p) or issubclass(t, C._Pointer), (name, decl)
            else:
                assert C.sizeof(t) == C.sizeof(widths[base]), (name, decl)
        ret = ret.strip()
        if "*" in ret:
            assert res in (C.c_void_p, C.c_char_p), name
        elif ret == "void":
            assert res is None, name
        else:
            assert res is C.c_int, name
