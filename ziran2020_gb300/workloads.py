"""Seeded families of synthetic scenes: the many-scene batch and the request stream of the serving loop.

Elastic-box family: a corotated cube over a sticky ground at dx = 1/64 with N particles (8 per cell, cube
side = round((N/8)^(1/3)) cells; cubes wider than 0.5 m use a finer dx instead), E ~ U(5e3, 5e4) Pa, centre ~ U[0.3, 0.7]^3 (moved inwards when the cube
would leave [0.1, 0.9]), v0 ~ U[-1, 1]^3 m/s. AnisoMPM-slab family: the 0.5 x 0.1 x 0.5 m slab with its
resolution chosen so that it holds about N particles.
"""
import math

import numpy as np

from . import RECIPE_ANISO_SLAB, RECIPE_ELASTIC_BOX, recipe, recipe_count


def elastic_family(rng, n_particles, dx=1 / 64, dt=1e-4):
    cells = max(2, int(round((n_particles / 8) ** (1 / 3))))
    if cells * dx > 0.5:  # keep the cube inside the unit box: refine the grid instead of growing the cube
        dx = 1 / math.ceil(cells / 0.5)
    side = cells * dx
    lo, hi = 0.1 + side / 2, 0.9 - side / 2
    center = [float(np.clip(c, lo, hi)) for c in rng.uniform(0.3, 0.7, 3)]
    return recipe(RECIPE_ELASTIC_BOX, seed=int(rng.integers(1 << 62)), dx=dx, dt=dt, size=(side, side, side), center=center,
                  velocity=[float(v) for v in rng.uniform(-1.0, 1.0, 3)], E=float(rng.uniform(5e3, 5e4)))


def slab_family(rng, n_particles, dt=5e-5):
    # 0.5 x 0.1 x 0.5 m at dx = 1/128 holds 425,984 particles; scale the resolution to reach n
    dx = (1 / 128) * (425984 / n_particles) ** (1 / 3)
    dx = 1 / max(16, round(1 / dx))
    return recipe(RECIPE_ANISO_SLAB, seed=int(rng.integers(1 << 62)), dx=dx, l0=0.5 * dx, dt=dt)


def log_uniform(rng, lo, hi):
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def batch_recipes(seed=20200713, count=256, n_min=5000, n_max=400000):
    """The many-scene batch: `count` elastic boxes with log-uniform particle counts."""
    rng = np.random.default_rng(seed)
    return [elastic_family(rng, log_uniform(rng, n_min, n_max)) for _ in range(count)]


def request_stream(seed, count, n_min=10000, n_max=2000000, steps_min=50, steps_max=500):
    """Serving requests: (recipe, substeps) pairs, each from the elastic or the AnisoMPM family."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = log_uniform(rng, n_min, n_max)
        r = elastic_family(rng, n) if rng.random() < 0.5 else slab_family(rng, n)
        out.append((r, int(rng.integers(steps_min, steps_max + 1))))
    return out


def total_particles(recipes):
    return sum(recipe_count(r) for r in recipes)
