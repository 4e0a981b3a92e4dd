"""Generate tests/golden/eoclover_4x4x4x4.npz: golden vectors of the even-odd clover solve.

The oracle (the FP64 restatement of Chroma's operator and InvCG2) is run once on a seeded 4^4
configuration; the fixture records the result so that later oracle builds, on any host, and the
GPU library are checked against the same fixed numbers:

- the action: Kappa 0.115, clovCoeff 1.2, hot links (eps 0.3, seed 2024), boundary (1, 1, 1, -1);
- ``plaquette``: plaquette and link trace of those links (a check that the seeded generator still
  gives the same field);
- ``src``: a Gaussian source on the odd sites (numpy PCG64, seed 7);
- ``meo``, ``meo_dag``: M~ src and M~^dag src (eoprec_clover_linop_w.cc:142-187);
- ``msym``: M_s src, the symmetric operator 1 - 1/4 A_oo^-1 D_oe A_ee^-1 D_eo
  (seoprec_clover_linop_w.cc:145-187);
- ``meo_tw``: M~ src with a twisted-mass term TwistedM = 0.05 (eoprec_clover_linop_w.cc:174-184);
- ``psi``: the solution of M~ psi = src by CGNE to a relative residual of 1e-13 (invcg2.cc:70-232);
- ``logdet_even``, ``logdet_odd``: sum of log|d| of the clover blocks' LDL^dag factors.
Spinors hold the odd sites only, in increasing site index ``x + Lx*(y + Ly*(z + Lz*t))``.

Usage:  python tests/golden/make_oracle_fixture.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

DIMS = (4, 4, 4, 4)
KAPPA, CSW, EPS, SEED, SRC_SEED = 0.115, 1.2, 0.3, 2024, 7
TWISTED_M = 0.05
PATH = os.path.join(HERE, "eoclover_4x4x4x4.npz")


def odd_sites(dims):
    s = np.arange(int(np.prod(dims)))
    x = s % dims[0]
    y = (s // dims[0]) % dims[1]
    z = (s // (dims[0] * dims[1])) % dims[2]
    t = s // (dims[0] * dims[1] * dims[2])
    return s[(x + y + z + t) % 2 == 1]


def links(orc):
    """The fixture's BC-applied links, rebuilt from the seed."""
    return orc.apply_bc(DIMS, orc.gauge_hot(DIMS, EPS, SEED), (1, 1, 1, -1))


def source():
    rng = np.random.default_rng(SRC_SEED)
    n = len(odd_sites(DIMS))
    return rng.standard_normal((n, 12)) + 1j * rng.standard_normal((n, 12))


def full(odd_part):
    """Odd-site spinor -> full-lattice (V, 12) array, zero on the even sites."""
    out = np.zeros((int(np.prod(DIMS)), 12), dtype=np.complex128)
    out[odd_sites(DIMS)] = odd_part
    return out


def main():
    from oracle import Oracle, OracleOp
    from oracle import oracle as O
    orc = Oracle()
    u = links(orc)
    op = OracleOp(DIMS, u, 1 / (2 * KAPPA) - 4, CSW)
    odd = odd_sites(DIMS)
    src = source()
    meo = op.apply(O.OP_MEO, full(src), +1, 1)[odd]
    meo_dag = op.apply(O.OP_MEO, full(src), -1, 1)[odd]
    msym = op.apply(O.OP_SYM, full(src), +1, 1)[odd]
    tw = OracleOp(DIMS, u, 1 / (2 * KAPPA) - 4, CSW, twisted_m=TWISTED_M)
    meo_tw = tw.apply(O.OP_MEO, full(src), +1, 1)[odd]
    psi, res = op.solve(full(src), solver=O.SOLVER_CG, rsd=1e-13, maxit=10000)
    np.savez_compressed(PATH, dims=np.array(DIMS, dtype=np.int32), kappa=KAPPA, csw=CSW, eps=EPS, seed=SEED,
                        src_seed=SRC_SEED, plaquette=np.array(orc.plaquette(DIMS, u), dtype=np.float64),
                        src=src, meo=meo, meo_dag=meo_dag, msym=msym, meo_tw=meo_tw, psi=psi[odd], rel_resid=res["rel_resid"],
                        logdet_even=op.logdet_even(), logdet_odd=op.logdet_odd())
    print(PATH, res)


if __name__ == "__main__":
    main()
