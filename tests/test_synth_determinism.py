"""The seeded geometry generators give the same geometry on every host.

Hashes of the sparse-block output (block coordinates, fluid masks, link records
and cut distances) committed here were produced on an x86_64 host and on the
aarch64 GPU host alike.  Two host dependences were removed to get there: the C
library's sin / cos / exp / cbrt (replaced by the generators' own functions made
of IEEE +, -, *, / and sqrt) and two random draws made inside one argument list
(whose evaluation order the two compilers choose differently).
"""
import hashlib

import numpy as np
import pytest

from hemelb_gb300.lbm import SyntheticGeometry

EXPECTED = {
    "tree_256": (444764, "864fcf525dee241c"),
    "bifurcation": (1464963, "52cbde4c48076699"),
    "ensemble_64": (4947705, "19c9394a0ea010d4"),
    "forest_6": (222966063, "8c2623fc90d707c7"),
}

MAKERS = {
    "tree_256": lambda: SyntheticGeometry.tree(seed=7, box_sites=256, n_roots=2, depth=5, root_radius=12.0),
    "bifurcation": lambda: SyntheticGeometry.bifurcation(1234, 24.0, 200.0, 2.5, 19, True),
    "ensemble_64": lambda: SyntheticGeometry.ensemble(2024, 64),
    # the benchmark's forest
    "forest_6": lambda: SyntheticGeometry.tree(seed=7, box_sites=1280, n_roots=6, depth=7, root_radius=60.0),
}


def _hash(g):
    m = hashlib.sha256()
    for a in (g.block_coords, g.fluid_mask, g.link_site, g.wall_mask, g.iolet_mask, g.iolet_id, g.site_type):
        m.update(np.ascontiguousarray(a).tobytes())
    if g.cut_distance is not None:
        m.update(np.ascontiguousarray(g.cut_distance).tobytes())
    return m.hexdigest()[:16]


@pytest.mark.parametrize("name", sorted(EXPECTED))
def test_generator_output_is_host_independent(name):
    g = MAKERS[name]()
    try:
        assert (int(g.n_fluid), _hash(g)) == EXPECTED[name]
    finally:
        g.close()
