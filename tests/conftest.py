import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def tatom(x, y, z, element="C", charge=0.0, name="CA", resseq=1, serial=1, chain="A",
              vdw_radius=1.7, epsilon=-0.1, rmin2=2.0):
    """The reference tests' create_test_atom (src/fitness.rs:308-330): every
    atom has serial 1, epsilon -0.1, Rmin/2 2.0 and radius 1.7 unless given."""
    return dict(x=x, y=y, z=z, element=element, charge=charge, name=name, resseq=resseq,
                serial=serial, chain=chain, vdw_radius=vdw_radius, epsilon=epsilon, rmin2=rmin2)


def make_mol(atoms):
    from gdock_gb300.pdb import Molecule
    n = len(atoms)
    g = lambda k, dt: np.array([a[k] for a in atoms], dtype=dt)
    return Molecule(
        serial=g("serial", np.int32), name=[a["name"] for a in atoms], altloc=[" "] * n,
        resname=["ALA"] * n, chainid=[a["chain"] for a in atoms], resseq=g("resseq", np.int16),
        icode=[" "] * n, x=g("x", np.float64), y=g("y", np.float64), z=g("z", np.float64),
        occupancy=np.ones(n, np.float32), tempfactor=np.zeros(n, np.float32),
        element=[a["element"] for a in atoms], charge=g("charge", np.float64),
        vdw_radius=g("vdw_radius", np.float64), epsilon=g("epsilon", np.float64),
        rmin2=g("rmin2", np.float64), eps_1_4=g("epsilon", np.float64), rmin2_1_4=g("rmin2", np.float64))


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc
    orc.build()
    return orc
