"""Writes tests/golden/sphdiffsemiinf.npz from the reference's analytic
fixture examples/meshtest/sphdiffsemiinf.mat: the diffusion solution of a
10 mm sphere (mua 0.05, mus' 0.5) in a 60 mm slab (mua 0.002, mus' 0.99),
source 30 mm below the sphere centre on its axis, on the plane y = 0 about the
sphere centre (x = -22:0.8:22, z = -30:0.8:10 mm), made by the reference as
sphdiffusionslab(0,0,60,-22:0.8:22,0,-30:0.8:10) (examples/meshtest/plotmmcsph.m:27-28).
Needs the reference tree, so it runs in the development container only; its
location comes from the command line or the MMC_REFERENCE environment
variable.

  MMC_REFERENCE=path/to/mmc python tests/golden/make_sphere_golden.py
"""
import os
import sys

import numpy as np
import scipy.io as sio

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref=None):
    ref = ref or os.environ.get("MMC_REFERENCE")
    if not ref or not os.path.isdir(os.path.join(ref, "examples")):
        sys.exit("set MMC_REFERENCE (or pass the path) to the reference MMC checkout")
    d = sio.loadmat(os.path.join(ref, "examples", "meshtest", "sphdiffsemiinf.mat"))
    phi = d["phi_ana"]
    assert np.abs(phi.imag).max() < 1e-12 * np.abs(phi.real).max()   # continuous wave: real
    np.savez_compressed(os.path.join(HERE, "sphdiffsemiinf.npz"), x=d["xa"][:, 0].astype(np.float64),
                        z=d["za"][0, :].astype(np.float64), phi=phi.real.astype(np.float64))


if __name__ == "__main__":
    main(*sys.argv[1:])
