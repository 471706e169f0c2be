"""Generate the golden fixtures in tests/golden/ from the reference's own plain
kernels run on the CPU (oracle/_ref/, built by `make -C oracle ref` from the
reference tree).  Each fixture holds the reference's fields after STEPS steps
from the reference's own initial state, as float64, at the reference's
compile-time size 512x512:

  kobayashi_ref.npz    snowflake/paras/para2.h, snowflake/function.h:5-60 (also at EARLY steps)
  graingrowth_ref.npz  graingrowth/paras/para1.h, graingrowth/function.h:5-30
  sintering_ref.npz    sintering/paras/para5.h, sintering/function.h:51-159

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import oracle_bind as ob  # noqa: E402

N = 512
STEPS = 40
EARLY = 8  # Kobayashi snapshot before any zero-gradient point is reached


def main():
    for name in ("snowflake", "graingrowth", "sintering"):
        if not ob.ref_available(name):
            raise SystemExit(f"oracle/_ref/libref_{name}.so missing: run `make -C oracle ref`")
    R = ob.ref_lib("snowflake")
    phi = np.zeros((N, N)); T = np.zeros((N, N))
    R.ref_snowflake_init(ob.ptr(phi), ob.ptr(T))
    R.ref_snowflake_steps(ob.ptr(phi), ob.ptr(T), EARLY)
    phi_early, T_early = phi.copy(), T.copy()
    R.ref_snowflake_steps(ob.ptr(phi), ob.ptr(T), STEPS - EARLY)
    np.savez_compressed(os.path.join(HERE, "kobayashi_ref.npz"), phi=phi, T=T, steps=STEPS,
                        phi_early=phi_early, T_early=T_early, early=EARLY,
                        params=ob.ref_params("snowflake", 14))

    R = ob.ref_lib("graingrowth")
    e1 = np.zeros((N, N)); e2 = np.zeros((N, N))
    R.ref_gg_init(ob.ptr(e1), ob.ptr(e2))
    R.ref_gg_steps(ob.ptr(e1), ob.ptr(e2), STEPS)
    np.savez_compressed(os.path.join(HERE, "graingrowth_ref.npz"), eta1=e1, eta2=e2, steps=STEPS,
                        params=ob.ref_params("graingrowth", 8))

    pr = ob.ref_params("sintering", 15)
    c, s1, s2 = ob.sint_init_two(N, N, pr[12], pr[13], pr[10], pr[14], pr[11])
    R = ob.ref_lib("sintering")
    R.ref_sint_steps(ob.ptr(c), ob.ptr(s1), ob.ptr(s2), STEPS)
    np.savez_compressed(os.path.join(HERE, "sintering_ref.npz"), c=c, eta1=s1, eta2=s2, steps=STEPS,
                        params=pr)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
