"""Triangles per marching-cubes case (UWW_CASE_NTRI of csrc/mc_tables.h), for
host-side consumers of a build's per-cell cases."""
import re
from pathlib import Path

import numpy as np

_HDR = Path(__file__).resolve().parent / "csrc" / "mc_tables.h"


def _table(name):
    m = re.search(name + r"\[256\]\s*=\s*\{(.*?)\};", _HDR.read_text(), re.S)
    return np.array([int(v, 0) for v in re.findall(r"0x[0-9a-f]+|\d+", m.group(1))], np.int64)


CASE_NTRI = _table("UWW_CASE_NTRI")
