// sgi_slots.cpp - C ABI of include/sgi_slots.h: the shadow-atlas slot cache.
//
// Free slots are a FIFO list in (atlas, layer) order; lights holding a slot are
// kept in the order they were given it (the eviction order), with a hash map
// from light id to its slot and its place in that order, so every call is O(1).
#include <cstdint>
#include <iterator>
#include <list>
#include <new>
#include <unordered_map>

#include "../../include/sgi_slots.h"

struct sgi_slot_cache {
    struct Held {
        sgi_atlas_entry slot;
        std::list<uint64_t>::iterator order;
    };
    std::list<sgi_atlas_entry> free_slots;
    std::list<uint64_t> order;                  // oldest assignment first
    std::unordered_map<uint64_t, Held> held;
    int32_t capacity = 0;
};

extern "C" {

sgi_status sgi_slot_cache_create(int32_t num_slots, int32_t slots_per_atlas, int32_t max_atlases,
                                 sgi_slot_cache** out) {
    if (!out || num_slots < 1 || slots_per_atlas < 1 || max_atlases < 1) return SGI_ERR_ARG;
    *out = nullptr;
    sgi_slot_cache* c = new (std::nothrow) sgi_slot_cache;
    if (!c) return SGI_ERR_OOM;
    // atlases of slots_per_atlas layers, the last one holding the remainder
    int32_t remaining = num_slots;
    for (int32_t a = 0; a < max_atlases && remaining > 0; ++a) {
        const int32_t layers = remaining < slots_per_atlas ? remaining : slots_per_atlas;
        for (int32_t l = 0; l < layers; ++l) c->free_slots.push_back(sgi_atlas_entry{a, l});
        remaining -= layers;
    }
    c->capacity = (int32_t)c->free_slots.size();
    *out = c;
    return SGI_OK;
}

sgi_status sgi_slot_cache_destroy(sgi_slot_cache* cache) {
    if (!cache) return SGI_ERR_ARG;
    delete cache;
    return SGI_OK;
}

sgi_status sgi_slot_cache_get(sgi_slot_cache* c, uint64_t light, sgi_atlas_entry* slot, int32_t* assigned,
                              uint64_t* evicted) {
    if (!c || !slot || light == SGI_NO_LIGHT) return SGI_ERR_ARG;
    if (assigned) *assigned = 0;
    if (evicted) *evicted = SGI_NO_LIGHT;
    auto it = c->held.find(light);
    if (it != c->held.end()) {
        *slot = it->second.slot;
        return SGI_OK;
    }
    sgi_atlas_entry s;
    if (!c->free_slots.empty()) {
        s = c->free_slots.front();
        c->free_slots.pop_front();
    } else {
        if (c->order.empty()) return SGI_ERR_STATE;   // no capacity (cannot happen: capacity >= 1)
        const uint64_t oldest = c->order.front();
        c->order.pop_front();
        auto o = c->held.find(oldest);
        s = o->second.slot;
        c->held.erase(o);
        if (evicted) *evicted = oldest;
    }
    c->order.push_back(light);
    try {
        c->held.emplace(light, sgi_slot_cache::Held{s, std::prev(c->order.end())});
    } catch (...) {
        c->order.pop_back();
        c->free_slots.push_front(s);
        return SGI_ERR_OOM;
    }
    *slot = s;
    if (assigned) *assigned = 1;
    return SGI_OK;
}

sgi_status sgi_slot_cache_remove(sgi_slot_cache* c, uint64_t light) {
    if (!c || light == SGI_NO_LIGHT) return SGI_ERR_ARG;
    auto it = c->held.find(light);
    if (it == c->held.end()) return SGI_OK;
    c->free_slots.push_back(it->second.slot);
    c->order.erase(it->second.order);
    c->held.erase(it);
    return SGI_OK;
}

sgi_status sgi_slot_cache_find(const sgi_slot_cache* c, uint64_t light, sgi_atlas_entry* slot) {
    if (!c || !slot || light == SGI_NO_LIGHT) return SGI_ERR_ARG;
    auto it = c->held.find(light);
    if (it == c->held.end()) return SGI_ERR_STATE;
    *slot = it->second.slot;
    return SGI_OK;
}

int32_t sgi_slot_cache_capacity(const sgi_slot_cache* c) { return c ? c->capacity : 0; }
int32_t sgi_slot_cache_free(const sgi_slot_cache* c) { return c ? (int32_t)c->free_slots.size() : 0; }
int32_t sgi_slot_cache_used(const sgi_slot_cache* c) { return c ? (int32_t)c->held.size() : 0; }

}  // extern "C"
