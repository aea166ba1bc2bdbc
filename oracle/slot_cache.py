"""Oracle (test infrastructure): the shadow-atlas slot bookkeeping of
StratusGFX's RendererBackend, restated from the reference so the C ABI's
slot cache (include/sgi_slots.h) can be checked against it.

- CreateShadowMap3DCache_ (Source/Engine/StratusRendererBackend.cpp:2397-2449):
  atlases of MAX_TOTAL_SHADOWS_PER_ATLAS layers (the last one the remainder), at
  most MAX_TOTAL_SHADOW_ATLASES, every (atlas, layer) pushed to the free list in
  order.
- GetOrAllocateShadowMapForLight_ (:2606-2632): a light with a slot gets it
  back (the LRU refresh at :2630 is commented out); otherwise the free list's
  front, or the slot of the light evicted by EvictOldestLightFromShadowMapCache_
  (:2657-2666: the front of cachedLights); the light is appended to cachedLights
  (AddLightToShadowMapCache_, :2673-2679).
- RemoveLightFromShadowMapCache_ (:2681-2693): the slot goes to the back of the
  free list and the light leaves cachedLights (EvictLightFromShadowMapCache_,
  :2640-2655).
"""
from __future__ import annotations


class SlotCacheModel:
    def __init__(self, count: int, per_atlas: int = 320, max_atlases: int = 14):
        self.free: list[tuple[int, int]] = []
        remaining, atlas = count, 0
        while remaining > 0 and atlas < max_atlases:
            tmp = remaining - per_atlas
            entries = remaining if tmp < 0 else per_atlas
            remaining = tmp
            self.free += [(atlas, layer) for layer in range(entries)]
            atlas += 1
        self.capacity = len(self.free)
        self.cached: list[int] = []              # cachedLights, oldest first
        self.slots: dict[int, tuple[int, int]] = {}

    def get(self, light: int):
        """(slot, assigned, evicted light or None)."""
        if light in self.slots:
            return self.slots[light], False, None
        evicted = None
        if self.free:
            slot = self.free.pop(0)
        else:
            evicted = self.cached.pop(0)
            slot = self.slots.pop(evicted)
        self.slots[light] = slot
        self.cached.append(light)
        return slot, True, evicted

    def remove(self, light: int):
        if light not in self.slots:
            return
        self.free.append(self.slots.pop(light))
        self.cached.remove(light)
