"""Autofocus (GetAutoFocusDistance, Source/autofocus.cuh:26-62) in the CPU
oracle.  The reference's kernel file does not compile (it names
ScatterEvent::Volume and Cuda::Allocate, which do not exist), so the oracle
restates it from its text; its march is the pinned fixed-step march."""
import numpy as np

import oracle_lib as OL

S = OL.PKG.scenes
AF_VIEW = 0x41F0C05E


def lanes(seed, w, u, v):
    return OL.seed_lanes(seed, AF_VIEW, v * w + u, 0)


def test_autofocus_hits_the_volume_front():
    orc = OL.load_oracle()
    sc = S.scene_c1(res=64, film=(64, 64))
    h = OL.SceneHandle(orc, sc)
    try:
        d = orc.autofocus(h.h, 32, 32, *lanes(1, 64, 32, 32))
        # camera at (0, -2, 0) looking at the unit-box volume: the blobs lie
        # between the front face (distance 1.5) and the back face (2.5)
        assert 1.5 < d < 2.5
        assert d == orc.autofocus(h.h, 32, 32, *lanes(1, 64, 32, 32))       # deterministic
        # a corner pixel whose rays miss the volume: the invalid event's
        # position is the origin, so the distance is |camera| = 2
        c = orc.autofocus(h.h, 0, 0, *lanes(1, 64, 0, 0))
        assert np.float32(c) == np.float32(2.0)
    finally:
        h.close()
