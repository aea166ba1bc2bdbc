/*
 * sgi_slots.h - the shadow-atlas slot cache of the lights whose cube maps the
 * stage samples (host only, no device work).
 *
 * Replaces RendererBackend's ShadowMapCache bookkeeping
 * (StratusRendererBackend.h:501-515; CreateShadowMap3DCache_,
 * StratusRendererBackend.cpp:2397-2449; GetOrAllocateShadowMapForLight_,
 * :2606-2632; EvictOldestLightFromShadowMapCache_, :2657-2666;
 * RemoveLightFromShadowMapCache_, :2681-2693). The engine keeps one cache for
 * the VPLs and one for the shadow-casting point lights (GetSmapCacheForLight_,
 * :2695-2697) and passes the slots it returns with each light
 * (sgi_set_lights, sgi_set_shadow_point_lights).
 *
 * Semantics (as the reference's):
 *   - the free slots are (atlas 0, layer 0 .. n0-1), (atlas 1, ...), ... with
 *     at most slots_per_atlas layers per atlas and at most max_atlases atlases;
 *   - a lookup of a light that holds a slot returns it and changes nothing
 *     (the reference's recency update is disabled: eviction order is the order
 *     in which lights were given their slots);
 *   - a light without a slot takes the first free slot; with none free, the
 *     light that was given its slot longest ago loses it and the new light
 *     takes that slot;
 *   - removing a light returns its slot to the end of the free list.
 */
#ifndef SGI_SLOTS_H_
#define SGI_SLOTS_H_

#include "sgi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sgi_slot_cache sgi_slot_cache;

#define SGI_NO_LIGHT ((uint64_t)0xffffffffffffffffull)

/* num_slots >= 1 slots, slots_per_atlas >= 1 layers per atlas (the reference:
 * 320), max_atlases >= 1 (the reference: 14); the capacity is
 * min(num_slots, slots_per_atlas * max_atlases). */
sgi_status sgi_slot_cache_create(int32_t num_slots, int32_t slots_per_atlas, int32_t max_atlases,
                                 sgi_slot_cache** out);
sgi_status sgi_slot_cache_destroy(sgi_slot_cache* cache);
/* The slot of `light` (any id but SGI_NO_LIGHT), assigning one if it has none.
 * *assigned = 1 when the slot was assigned by this call (its cube map must be
 * rendered), else 0; *evicted = the light that lost the slot, or
 * SGI_NO_LIGHT. assigned and evicted may be NULL. */
sgi_status sgi_slot_cache_get(sgi_slot_cache* cache, uint64_t light, sgi_atlas_entry* slot, int32_t* assigned,
                              uint64_t* evicted);
/* Releases the slot of `light` (nothing happens if it holds none). */
sgi_status sgi_slot_cache_remove(sgi_slot_cache* cache, uint64_t light);
/* The slot `light` holds without assigning one: SGI_OK, or SGI_ERR_STATE if none. */
sgi_status sgi_slot_cache_find(const sgi_slot_cache* cache, uint64_t light, sgi_atlas_entry* slot);
/* Capacity, slots free, lights holding a slot. */
int32_t sgi_slot_cache_capacity(const sgi_slot_cache* cache);
int32_t sgi_slot_cache_free(const sgi_slot_cache* cache);
int32_t sgi_slot_cache_used(const sgi_slot_cache* cache);

#ifdef __cplusplus
}
#endif

#endif /* SGI_SLOTS_H_ */
