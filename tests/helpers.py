"""Shared comparison helpers for the parity tests."""
from __future__ import annotations

from pathlib import Path

import numpy as np

from underwaterworld_gb300 import abi
from underwaterworld_gb300.chunk import make_descs

GOLDEN = Path(__file__).resolve().parent / "golden"

# Tolerances.  Positions, indices, cases, counts and flags are compared
# bit-exactly in the parity (exact) build.  Colours pass through powf, whose
# last-bit rounding differs between the CPU libm and CUDA: absolute 2e-6 on
# values in [0, 1].  Normals: 1e-6 relative (they are unit vectors, so absolute).
COLOR_ATOL = 2e-6
NORMAL_ATOL = 1e-6
RECORD_FIELDS = ("num_verts", "num_inds", "vert_offset", "ind_offset", "flags", "num_active_cells")


def load_golden(name: str):
    z = np.load(GOLDEN / "mc_known_answers.npz")
    d = {k.split("/", 1)[1]: z[k] for k in z.files if k.startswith(name + "/")}
    d["descs"] = make_descs(d["pos"], d["cells"])
    return d


def assert_records_equal(a, b):
    for f in RECORD_FIELDS:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f"record field {f}")


def assert_batches_equal(got, want, exact_positions=True, check_colors=True, check_normals=True):
    """got/want are MeshBatch results of the same descriptors."""
    assert_records_equal(got.records, want.records)
    np.testing.assert_array_equal(got.inds, want.inds, err_msg="index buffers")
    if exact_positions:
        np.testing.assert_array_equal(got.verts["pos"], want.verts["pos"], err_msg="vertex positions")
    else:
        np.testing.assert_allclose(got.verts["pos"], want.verts["pos"], rtol=1e-6, atol=1e-5)
    if check_colors:
        np.testing.assert_allclose(got.verts["color"], want.verts["color"], rtol=0, atol=COLOR_ATOL)
    if check_normals and got.normals is not None and want.normals is not None:
        np.testing.assert_allclose(got.normals, want.normals, rtol=0, atol=NORMAL_ATOL)
    if got.cases is not None and want.cases is not None:
        np.testing.assert_array_equal(got.cases, want.cases, err_msg="cell cases")
    np.testing.assert_array_equal(got.totals[:3], want.totals[:3], err_msg="totals")


def params_for_samples(iso_level: float, outputs: int = abi.UWW_OUT_COLOR | abi.UWW_OUT_CASES):
    p = abi.reference_params()
    p.iso_level = float(iso_level)
    p.outputs = outputs
    return p


def relayout(descs):
    """Descriptors of a subset, with their per-cell and per-sample offsets re-packed."""
    return make_descs(descs["pos"], descs["cells"])


def flipped_cells(cases_a: np.ndarray, cases_b: np.ndarray) -> int:
    return int(np.count_nonzero(cases_a != cases_b))
