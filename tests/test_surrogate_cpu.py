"""Host-side pieces of the warm-start surrogate: the symmetry augmentation maps a
velocity field to the field of the mirrored / swapped geometry, and samples are
seeded and reproducible."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from hemelb_gb300 import surrogate as S  # noqa: E402


def _field(B):
    i = np.arange(B, dtype=np.float64) - (B - 1) / 2.0
    X, Y, Z = np.meshgrid(i, i, i, indexing="ij")
    # an arbitrary smooth vector field u(x, y, z) and scalar p(x, y, z)
    u = np.stack([np.sin(0.3 * X) + 0.1 * Y, np.cos(0.2 * Y) * X, 0.05 * Z + X * Y / 50.0], axis=-1)
    p = 0.01 * X + 0.02 * Y * Y + 0.03 * Z
    return X, Y, Z, u, p


@pytest.mark.parametrize("code", range(8))
def test_augmentation_is_the_symmetry_of_the_field(code):
    B = 8
    X, Y, Z, u, p = _field(B)
    g = S.Grids(1, B, device="cpu")
    g.target[0, ..., :3] = torch.from_numpy(u).float()
    g.target[0, ..., 3] = torch.from_numpy(p).float()
    g.mask[0] = torch.from_numpy(((X + Y) > 0).astype(np.uint8))
    t, m = g.targets([0], code)
    # the transformed field evaluated at the voxel centres, in closed form
    sx = -1.0 if code & 1 else 1.0
    sy = -1.0 if code & 2 else 1.0
    if code & 4:  # new (x, y) = old (y, x) after the mirrors
        Xo, Yo = sx * Y, sy * X
    else:
        Xo, Yo = sx * X, sy * Y
    _, _, _, uo, po = _field(B)
    # look up the old field at the old position of each new voxel
    idx = lambda c: np.rint(c + (B - 1) / 2.0).astype(int)
    ix, iy, iz = idx(Xo), idx(Yo), idx(Z)
    vo = uo[ix, iy, iz]
    vx, vy = sx * vo[..., 0], sy * vo[..., 1]
    if code & 4:
        vx, vy = vy, vx
    expect = np.stack([vx, vy, vo[..., 2], po[ix, iy, iz]], axis=-1)
    assert np.allclose(t[0, ..., :4].numpy(), expect, atol=1e-6)
    assert np.array_equal(m[0].numpy(), (((X + Y) > 0).astype(np.float32))[ix, iy, iz])
    assert torch.count_nonzero(t[..., 4:]) == 0


def test_samples_are_seeded():
    a = [S.Sample.draw(i) for i in range(20)]
    b = [S.Sample.draw(i) for i in range(20)]
    assert a == b
    assert len({s.seed for s in a}) == 20
    assert {s.kind for s in a} == {0, 1}
    assert all(0.7 <= s.tau <= 1.0 and 5e-4 <= s.drho <= 3e-3 for s in a)
    assert S.Sample.draw(0, box=48).box == 48


def test_vessel_box_geometry_and_reference_speed():
    smp = S.Sample.draw(3, box=48)
    g = smp.geometry()
    assert g.box_shape() == (48, 48, 48)
    fl = g.fluid_grid()
    assert fl.sum() == g.n_fluid
    sd = g.signed_distance()
    assert ((sd > 0) == fl).mean() > 0.99  # the distance sign agrees with the voxelisation
    r_in = g.iolet(False, 0)[2]
    nu = (smp.tau - 0.5) / 3.0
    assert abs(smp.u_ref(g) - smp.drho / 3.0 / 48 * r_in ** 2 / (4 * nu)) < 1e-15
