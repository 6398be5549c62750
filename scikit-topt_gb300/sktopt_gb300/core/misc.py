"""Restart helper (sktopt/core/misc.py:8-22)."""
from __future__ import annotations

import os
import re


def find_latest_iter_file(data_dir: str):
    best, path = -1, None
    for f in os.listdir(data_dir):
        m = re.match(r"^(\d{6})-rho\.npz$", f)
        if m and int(m.group(1)) > best:
            best, path = int(m.group(1)), os.path.join(data_dir, f)
    if path is None:
        raise FileNotFoundError(f"no NNNNNN-rho.npz in {data_dir}")
    return best, path
