"""The analytic sphere-in-slab diffusion restatement (oracle/sphdiffusion.py)
against the reference's own analytic fixture (tests/golden/sphdiffsemiinf.npz,
from examples/meshtest/sphdiffsemiinf.mat)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
import sphdiffusion as sd  # noqa: E402


def test_sphere_in_slab_matches_reference_fixture():
    f = np.load(os.path.join(HERE, "golden", "sphdiffsemiinf.npz"))
    x, z = np.meshgrid(f["x"], f["z"], indexing="ij")
    phi = sd.slab(0.0, 0.0, 60.0, x, np.zeros_like(x), z)
    assert np.abs(phi.imag).max() < 1e-12 * np.abs(phi.real).max()
    np.testing.assert_allclose(phi.real, f["phi"], rtol=1e-9)


def test_homogeneous_sphere_reduces_to_the_point_source():
    """A sphere with the background's optical properties scatters nothing:
    the infinite-medium field is the free-space Green's function, inside and
    outside the sphere."""
    cfg = sd.SphereCfg(imua=0.002, imusp=0.990)
    x = np.array([0.0, 3.0, -5.0, 12.0, 0.0])
    z = np.array([0.0, -4.0, 8.0, 1.0, 25.0])
    y = np.zeros_like(x)
    phi = sd.infinite(x, y, z, cfg)
    np.testing.assert_allclose(phi, sd.incident(x, y, z, cfg), rtol=1e-8)


def test_homogeneous_semi_infinite_closed_form():
    """With a sphere of the background's properties the semi-infinite
    solution is the closed-form pair of image sources."""
    cfg = sd.SphereCfg(omua=0.005, omusp=0.99, imua=0.005, imusp=0.99)
    x = np.array([0.0, 5.0, 10.0, 0.0, 8.0, 3.0])
    z = np.array([-20.0, -15.0, -10.0, 0.0, -5.0, 12.0])
    phi = sd.semi_infinite(0.0, x, np.zeros_like(x), z, cfg)
    np.testing.assert_allclose(phi.real, sd.point_semi_infinite(0.0, 0.005, 0.99, x, 0.0, z + 30.0), rtol=1e-8)
    # an index-mismatched boundary (R > 0) moves the image source away and raises the fluence
    assert np.all(sd.point_semi_infinite(0.4, 0.005, 0.99, x, 0.0, z + 30.0) > phi.real)
