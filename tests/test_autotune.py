"""CPU: the batched form's autotuner (choice of render lanes and depth-slab schedule, cached per batch
shape) with a stand-in renderer and timer; the GPU timing itself is exercised by the bench."""

import json

from vkgs_gb300 import autotune


class _Cam:
    def __init__(self, w, h):
        self.width, self.height = w, h


class _Splats:
    count = 1000


class _Renderer:
    def __init__(self):
        self.lanes, self.slabs, self.calls = 0, (1024,), []

    def set_batch_lanes(self, n):
        self.lanes = n
        self.calls.append(("lanes", n))

    def set_slabs(self, ends):
        self.slabs = tuple(ends)
        self.calls.append(("slabs", tuple(ends)))

    def render_batched_checked(self, splats, cams, colors):
        self.calls.append(("checked", self.lanes))


def test_autotune_picks_the_fastest_pair_and_caches_it(tmp_path, monkeypatch):
    cams = [_Cam(640, 360), _Cam(1920, 1080)]
    # pretend 8 lanes with slabs (256, 1024) is fastest
    monkeypatch.setattr(autotune, "time_batch",
                        lambda r, s, c, col, reps=5: 1.0 + abs(r.lanes - 8) + (0 if r.slabs == (256, 1024) else 0.5))
    r = _Renderer()
    cache = tmp_path / "tune.json"
    choice = autotune.autotune_batched(r, _Splats(), cams, [None, None], cache=str(cache))
    assert (choice.lanes, choice.slabs) == (8, (256, 1024))
    assert (r.lanes, r.slabs) == (8, (256, 1024))
    assert r.calls[0] == ("lanes", max(autotune.LANES))  # capacity sized once with the most lanes
    key = autotune.batch_key(_Splats.count, cams)
    assert json.loads(cache.read_text())[key]["lanes"] == 8

    # a second call with the same batch shape reads the cache and times nothing
    monkeypatch.setattr(autotune, "time_batch", lambda *a, **k: (_ for _ in ()).throw(AssertionError("timed")))
    r2 = _Renderer()
    again = autotune.autotune_batched(r2, _Splats(), cams, [None, None], cache=str(cache))
    assert (again.lanes, again.slabs) == (8, (256, 1024)) and (r2.lanes, r2.slabs) == (8, (256, 1024))


def test_batch_key_ignores_view_order():
    a = autotune.batch_key(10, [_Cam(640, 360), _Cam(1920, 1080)])
    b = autotune.batch_key(10, [_Cam(1920, 1080), _Cam(640, 360)])
    assert a == b and a != autotune.batch_key(11, [_Cam(640, 360), _Cam(1920, 1080)])
