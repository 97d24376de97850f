"""Regenerate tests/golden/block_model_oracle.npz (run from the repo root).

The reference cannot be imported in the build container (its discretize /
pymatsolver dependencies are absent), so these fixtures are produced by the
CPU oracle (``oracle/``: the reference path restated on SciPy SuperLU) on the
32x32x16 block-model workload and pin the oracle against drift; the GPU
parity tests compare with them directly.
"""

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.dc3d import OracleDC3DNodal  # noqa: E402
from simpeg_gb300 import maps  # noqa: E402
from simpeg_gb300.workloads import block_model_survey  # noqa: E402


def main():
    mesh, sigma, survey, blocks = block_model_survey(seed=0)
    m = np.log(sigma)
    o = OracleDC3DNodal(mesh, survey, sigma_map=maps.ExpMap(mesh))
    o.set_model(m)
    f = o.fields()
    rng = np.random.default_rng(2024)
    v = rng.standard_normal(mesh.n_cells)
    w = rng.standard_normal(survey.nD)
    out = dict(
        m=m, v=v, w=w, blocks=np.array(blocks),
        dpred=o.dpred(f=f), jvec=o.Jvec(m, v, f=f), jtvec=o.Jtvec(m, w, f=f),
    )
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "block_model_oracle.npz"), **out)
    print({k: np.asarray(a).shape for k, a in out.items()})


if __name__ == "__main__":
    main()
