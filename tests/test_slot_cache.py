"""The shadow-atlas slot cache of the C ABI (host only) against the
restatement of the reference's bookkeeping: known sequences and a long
seeded sequence of lookups and removals."""
import ctypes as C
import os
import random
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle.slot_cache import SlotCacheModel  # noqa: E402
from stratusgfx_gb300 import abi  # noqa: E402


class Cache:
    def __init__(self, n, per_atlas=320, max_atlases=14):
        self.lib = abi.load()
        self.h = C.c_void_p()
        assert self.lib.sgi_slot_cache_create(n, per_atlas, max_atlases, C.byref(self.h)) == abi.SGI_OK

    def get(self, light):
        e, a, ev = abi.AtlasEntry(), C.c_int32(), C.c_uint64()
        assert self.lib.sgi_slot_cache_get(self.h, light, C.byref(e), C.byref(a), C.byref(ev)) == abi.SGI_OK
        return (e.index, e.layer), bool(a.value), (None if ev.value == abi.SGI_NO_LIGHT else ev.value)

    def remove(self, light):
        assert self.lib.sgi_slot_cache_remove(self.h, light) == abi.SGI_OK

    def close(self):
        assert self.lib.sgi_slot_cache_destroy(self.h) == abi.SGI_OK


def test_fifo_eviction_and_free_list_order():
    c = Cache(3, per_atlas=2)
    try:
        assert c.lib.sgi_slot_cache_capacity(c.h) == 3
        assert [c.get(k) for k in (10, 11, 12)] == [((0, 0), True, None), ((0, 1), True, None), ((1, 0), True, None)]
        assert c.get(11) == ((0, 1), False, None)          # a hit changes nothing
        assert c.get(13) == ((0, 0), True, 10)             # the oldest assignment is evicted
        c.remove(12)                                       # its slot goes to the free list
        assert c.lib.sgi_slot_cache_free(c.h) == 1 and c.lib.sgi_slot_cache_used(c.h) == 2
        assert c.get(14) == ((1, 0), True, None)
        assert c.get(15) == ((0, 1), True, 11)             # 11 was assigned before 13 and 14
        e = abi.AtlasEntry()
        assert c.lib.sgi_slot_cache_find(c.h, 10, C.byref(e)) == abi.SGI_ERR_STATE
        assert c.lib.sgi_slot_cache_find(c.h, 15, C.byref(e)) == abi.SGI_OK and (e.index, e.layer) == (0, 1)
    finally:
        c.close()


def test_capacity_is_capped_by_the_atlas_count():
    c = Cache(1000, per_atlas=64, max_atlases=3)
    try:
        assert c.lib.sgi_slot_cache_capacity(c.h) == 192
    finally:
        c.close()


def test_bad_arguments():
    lib = abi.load()
    h = C.c_void_p()
    assert lib.sgi_slot_cache_create(0, 320, 14, C.byref(h)) == abi.SGI_ERR_ARG
    assert lib.sgi_slot_cache_create(4, 0, 14, C.byref(h)) == abi.SGI_ERR_ARG
    c = Cache(2)
    try:
        e = abi.AtlasEntry()
        assert c.lib.sgi_slot_cache_get(c.h, abi.SGI_NO_LIGHT, C.byref(e), None, None) == abi.SGI_ERR_ARG
        assert c.lib.sgi_slot_cache_get(c.h, 5, C.byref(e), None, None) == abi.SGI_OK
    finally:
        c.close()


@pytest.mark.parametrize("n,per_atlas", [(7, 3), (40, 320), (700, 320)])
def test_matches_the_reference_bookkeeping(n, per_atlas):
    rng = random.Random(n)
    c = Cache(n, per_atlas=per_atlas)
    m = SlotCacheModel(n, per_atlas=per_atlas)
    try:
        assert c.lib.sgi_slot_cache_capacity(c.h) == m.capacity
        for _ in range(20000):
            light = rng.randrange(3 * n)
            if rng.random() < 0.2:
                c.remove(light)
                m.remove(light)
            else:
                assert c.get(light) == m.get(light)
        assert c.lib.sgi_slot_cache_used(c.h) == len(m.slots)
        assert c.lib.sgi_slot_cache_free(c.h) == len(m.free)
    finally:
        c.close()
