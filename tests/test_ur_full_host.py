"""DnsState.ur_full semantics without a GPU: a fake field stands in for the
handle and counts the plane copies."""
import numpy as np

from palinstrophy_gb300.turbo_simulator import _UrFull


class _FakeField:
    def __init__(self, M):
        self.M = M
        self.rdt = np.float32
        self.gen = 0
        self.copies = []

    def ur_into(self, comp, out):
        self.copies.append(comp)
        out[...] = (comp + 1) * 10 + self.gen
        return out


def test_planes_copy_once_per_change_and_one_at_a_time():
    f = _FakeField(6)
    ur = _UrFull(f)
    assert ur.shape == (3, 6, 6) and len(ur) == 3
    u = ur[0]
    assert f.copies == [0] and (u == 10).all()
    _ = ur[0, :, :]
    _ = ur[0]
    assert f.copies == [0]                       # cached until the field changes
    v = ur[1, 2:4, :]
    assert f.copies == [0, 1] and (v == 20).all()
    f.gen += 1                                   # a step
    assert (ur[0] == 11).all() and f.copies == [0, 1, 0]
    assert (u == 11).all()                       # earlier views see the refresh in place
    arr = np.asarray(ur)
    assert arr.shape == (3, 6, 6) and f.copies == [0, 1, 0, 1]


def test_display_plane_persists_and_is_not_refreshed():
    f = _FakeField(4)
    ur = _UrFull(f)
    ur.plane2()[...] = 7.0                       # what a display helper writes
    assert (ur[2, :, :] == 7.0).all()
    assert f.copies == []                        # plane 2 never comes from the device
    f.gen += 1
    assert (np.asarray(ur[2]) == 7.0).all()
    ur[2, :, :] = 3.0                            # callers may write it, as in the reference
    assert (ur[2] == 3.0).all()
