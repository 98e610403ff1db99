"""The scene configurations as data (no GPU): the batched view set is
uneven, reproducible and covers the eight sun elevations."""
import math

import pytest

from vcr import configs


def test_c4_view_set_is_uneven_and_covers_eight_suns():
    views = configs.c4_views(64, seed=1)
    sides = [w for _, w, h, _ in views]
    assert len(views) == 64 and all(w == h for _, w, h, _ in views)
    assert min(sides) >= 256 and max(sides) <= 1024 and len(set(sides)) > 32
    elev = {round(math.degrees(math.asin(-s[1])), 3) for _, _, _, s in views}
    assert len(elev) == 8 and min(elev) == pytest.approx(5.0) and max(elev) == pytest.approx(80.0)
    again = configs.c4_views(64, seed=1)
    assert [w for _, w, _, _ in again] == sides


def test_c4_cameras_look_at_the_cloud():
    for cam, w, h, _ in configs.c4_views(8, seed=2):
        pos = [cam.position[i] for i in range(3)]
        fwd = [cam.forward[i] for i in range(3)]
        to_centre = [0.0 - pos[0], 0.0 - pos[1], 0.5 - pos[2]]
        n = math.sqrt(sum(c * c for c in to_centre))
        assert sum(f * c / n for f, c in zip(fwd, to_centre)) > 0.999
        assert cam.half_width * 2 in (w, w - 1, w + 1)


def test_scene_digest_names_the_configuration():
    import dataclasses
    digests = {sc.digest() for sc in configs.ALL}
    assert len(digests) == len(configs.ALL)
    sc = configs.C5_NRC
    d = sc.digest()
    assert len(d) == 16 and int(d, 16) >= 0
    assert dataclasses.replace(sc).digest() == d
    assert dataclasses.replace(sc, seed=sc.seed + 1).digest() != d
    assert dataclasses.replace(sc, g=0.5).digest() != d
