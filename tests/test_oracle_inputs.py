"""CPU: the oracle's own seeded-input generator (used by the CPU baseline, which must not load the product
library) gives the library's recipe particles bit for bit, and its scene matches the library's recipe scene."""
import numpy as np
import pytest

import pyoracle as po
import ziran2020_gb300 as zr


@pytest.mark.parametrize("kind,over", [(zr.RECIPE_ELASTIC_BOX, dict(size=(0.125, 0.125, 0.125))),
                                       (zr.RECIPE_ANISO_SLAB, dict(dx=1 / 256, size=(0.05, 0.03, 0.04))),
                                       (zr.RECIPE_ANISO_SLAB, dict(size=(0.1, 0.05, 0.1), center=(0.43, 0.52, 0.61)))])
def test_oracle_inputs_equal_library_recipe(kind, over):
    kw = dict(over)
    r = zr.recipe(kind, seed=777, **{k: v for k, v in kw.items()})
    g = zr.recipe_generate(r)
    o, _ = po.seeded_inputs(kind, seed=777, **kw)
    assert len(o["m"]) == zr.recipe_count(r)
    for k in ("x", "v", "m", "V0", "F", "sigma_c"):
        assert np.array_equal(np.asarray(g[k]).reshape(o[k].shape), o[k]), k


def test_oracle_slab_scene_follows_library_scene_rules():
    """One substep of the oracle's slab scene equals one substep of the oracle fed with the library's
    recipe arrays and the test suite's scene rules (plates, materials, damage constants)."""
    import scenes

    dx = 1 / 128
    a, n = po.recipe_scene(1, 8, seed=11, size=(0.1, 0.05, 0.1))
    d = scenes.aniso_slab(size=(0.1, 0.05, 0.1), dx=dx, seed=11)
    assert n == len(d["m"])
    b = scenes.oracle_scene(d, 8)
    a.step(2)
    b.step(2)
    sa, sb = a.state(), b.state()
    for k in ("x", "v", "F", "d"):
        assert np.array_equal(sa[k], sb[k]), k
