import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
if REPO not in sys.path:
    sys.path.insert(0, REPO)

COSMO = dict(OmegaM=0.315, OmegaL=0.685, OmegaB=0.049, hhub=0.67, weos=-1.0, n_scal=0.96, sig8=0.83)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built extension")


def load_case(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def oracle_for_case(case, **over):
    """Oracle configured like the reference run that produced a golden case
    (keyword arguments override oracle configuration fields)."""
    from oracle import orc
    k, pk = orc.load_pk(os.path.join(GOLDEN, "pk_eh_nowiggle.txt"))
    reg = int(case["cfg_regular_nu"])
    cfg = dict(COSMO, r_smooth=float(case["cfg_r_smooth"]) if "cfg_r_smooth" in case else 2.0,
               n_grid=int(case["cfg_n_grid"]), n_side=int(case["cfg_n_side"]), seed=int(case["cfg_seed"]),
               regular_nu=reg)
    cfg.update(over)
    if reg:
        cfg.update(nu_min=float(case["cfg_nu_min"]), nu_max=float(case["cfg_nu_max"]),
                   n_nu=int(case["cfg_n_nu"]))
        return orc.Oracle(cfg, k, pk)
    edges = np.loadtxt(os.path.join(GOLDEN, "nutable_8.txt"))
    return orc.Oracle(cfg, k, pk, edges[:-1], edges[1:])


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import orc
    orc.build()
    return orc
