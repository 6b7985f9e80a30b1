"""The oracle still reproduces the committed golden fixtures (CPU only)."""
import glob
import os

import numpy as np
import pytest

from oracle import spe

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))


def load_case(path):
    d = dict(np.load(path, allow_pickle=False))
    d["convention"] = str(d["convention"])
    d["mode"] = str(d["mode"])
    return d


def oracle_physics(d):
    g = spe.Grid(tuple(int(v) for v in d["n"]), tuple(float(v) for v in d["L"]), d["convention"])
    rho_b = spe.cic_deposit(g, d["pos"], d["mass"]) if "pos" in d else None
    sched = d.get("tidal")
    dt = float(d["dt"])
    tidal = None
    if sched is not None:
        def tidal(t, sched=sched):
            return tuple(sched[int(round(t / dt))])
    phys = spe.Physics(poisson_coeff=float(d["c"]), kerr=float(d["kerr"]), absorb_alpha=float(d["alpha"]),
                       V_static=d.get("V"), rho_b=rho_b, tidal=tidal)
    return g, phys


@pytest.mark.parametrize("path", FILES, ids=[os.path.basename(f)[:-4] for f in FILES])
def test_oracle_reproduces_golden(path):
    d = load_case(path)
    g, phys = oracle_physics(d)
    psi = spe.run(d["psi0"], g, phys, float(d["dt"]), int(d["steps"]), mode=d["mode"])
    assert spe.rel_l2(psi, d["psi"]) < 1e-12


def test_golden_files_present():
    assert len(FILES) >= 4
