"""Loader of the reference-generated fixtures in tests/golden/ (see make_golden.py there)."""
from __future__ import annotations

import os

import numpy as np
import scipy.sparse as sp

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FULL_CASES = ["tri2d_n8_k1", "tri2d_n32_k1", "tri2d_n50_k1", "tri2d_n16_k2", "tet3d_n4_k1", "tet3d_n8_k1",
              "tet3d_n4_k2"]
HISTORY_CASES = ["tet3d_n16_k1", "tet3d_n32_k1", "tet3d_n64_k1"]


class Case:
    def __init__(self, name: str):
        self.name = name
        z = np.load(os.path.join(GOLDEN, name + ".npz"))
        self.z = z
        self.dim, self.n, self.k = int(z["dim"]), int(z["n"]), int(z["k"])
        self.bs = int(z["block_size"])
        self.levels = int(z["levels"])
        self.has_hierarchy = "A0_data" in z
        if self.has_hierarchy:
            self.As = []
            for l in range(self.levels):
                n = int(z["level_rows"][l])
                self.As.append(sp.csr_matrix((z[f"A{l}_data"], z[f"A{l}_indices"], z[f"A{l}_indptr"]), shape=(n, n)))
            self.Ps = [sp.csr_matrix((z[f"P{l}_data"], z[f"P{l}_indices"], z[f"P{l}_indptr"]),
                                     shape=tuple(int(v) for v in z[f"P{l}_shape"])) for l in range(self.levels - 1)]
            self.perms = [np.asarray(z[f"perm{l}"]) for l in range(self.levels)]
            self.b = np.asarray(z["b"])

    def __getitem__(self, key):
        return self.z[key]


def available(names):
    return [n for n in names if os.path.exists(os.path.join(GOLDEN, n + ".npz"))]
