"""Generate the golden vectors in this directory from the reference's own hot-path code.

The reference's common/ modules are translated to C (oracle/f90c.py), compiled with the
single-rank glue and run on a small seeded Weibel state; inputs and outputs are saved to
golden_weibel_16x12.npz.  Needs the reference source tree (WM_REFERENCE_COMMON, default: the
common/ directory of a checkout named "reference" beside this repository); the committed .npz is
what the tests read.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import reference as R  # noqa: E402
from tests.helpers import State  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden_weibel_16x12.npz"


def main():
    if not R.available():
        raise SystemExit("reference source tree not available")
    g = {}
    # one-routine vectors from a state with random fields and a random previous delta-B
    st = State(nx=16, ny=12, ppc=4, seed=77, field_amp=0.06, df_amp=1e-3)
    d = st.d
    ref = R.Reference(d, st.cfg.delt, st.cfg.charge, st.cfg.mass)
    g.update(nx=d.nx, ny=d.ny, np=d.np, nsp=d.nsp, delt=st.cfg.delt, q=st.cfg.charge, r=st.cfg.mass, c=1.0, delx=1.0,
             gfac=0.501, in_up=st.up, in_uf=st.uf, in_cumcnt=st.cumcnt, in_np2=st.np2, in_df=st.df, in_gp=st.gp)
    gp = st.gp.copy(order="F")
    assert ref.particle_solv(gp, st.up, st.uf, st.cumcnt) == 0
    g["push_gp"] = gp.copy()
    acc = st.gp.copy(order="F")
    assert ref.mom_accl(acc, st.up, st.uf, st.cumcnt) == 0
    g["accl_gp"] = acc
    ref.set_df(st.df)
    uf = st.uf.copy(order="F")
    assert ref.field_fdtd_i(uf, st.up, gp, st.cumcnt) == 0
    df, uj, gkl = ref.get_work()
    g.update(fdtd_uf=uf, fdtd_df=df, fdtd_uj=uj, fdtd_gkl=gkl)
    np2 = st.np2.copy(order="F")
    assert ref.bc_particle_x(gp, np2) == 0
    g["px_gp"] = gp.copy()
    assert ref.bc_particle_y(gp, np2) == 0
    g.update(py_gp=gp.copy(), py_np2=np2.copy())
    out = st.up.copy(order="F")
    cum = d.alloc_cumcnt()
    assert ref.sort_bucket(out, gp, cum, np2) == 0
    g.update(sort_up=out, sort_cumcnt=cum)
    mom = d.alloc_mom()
    assert ref.mom_nvt(mom, st.up, st.np2) == 0
    g["nvt_mom"] = mom.copy()
    assert ref.bc_mom(mom) == 0
    g["bcmom_mom"] = mom

    # five full steps of the seeded Weibel plasma from zero fields (fresh module state)
    st2 = State(nx=16, ny=12, ppc=4, seed=78)
    ref2 = R.Reference(st2.d, st2.cfg.delt, st2.cfg.charge, st2.cfg.mass)
    g.update(run_in_up=st2.up.copy(), run_in_uf=st2.uf.copy(), run_in_cumcnt=st2.cumcnt.copy(), run_in_np2=st2.np2.copy())
    for _ in range(5):
        assert ref2.step(st2.up, st2.gp, st2.uf, st2.cumcnt, st2.np2) == 0
    df2, uj2, _ = ref2.get_work()
    g.update(run_up=st2.up, run_uf=st2.uf, run_cumcnt=st2.cumcnt, run_np2=st2.np2, run_df=df2, run_uj=uj2)
    np.savez_compressed(OUT, **g)
    print(OUT, OUT.stat().st_size, "bytes")


if __name__ == "__main__":
    main()
