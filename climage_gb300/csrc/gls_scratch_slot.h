// gls_scratch_slot.h -- per-device cache of a static device array's address, keyed on the
// CUDA context the address was looked up in.  Host code only, no CUDA types: the caller
// supplies the id of the current context (cuCtxGetId; 0 when none is current) and a lookup
// that returns the address together with the id of the context it was looked up in.
#ifndef GLS_SCRATCH_SLOT_H
#define GLS_SCRATCH_SLOT_H

namespace gls {

struct ScratchSlot {
    unsigned long long ctx_id = 0;  // context of ptr (0: nothing looked up yet)
    void* ptr = nullptr;
};

// The cached address while `now` is the context it belongs to; otherwise (no context
// current yet, a device reset, another context) lookup(&id) runs again and its result
// replaces the cache.  A failed lookup (null address or id 0) returns null and leaves the
// cache as it was.
template <class Lookup>
inline void* scratch_slot_get(ScratchSlot& slot, unsigned long long now, Lookup&& lookup) {
    if (now != 0 && now == slot.ctx_id) return slot.ptr;
    unsigned long long id = 0;
    void* p = lookup(&id);
    if (!p || id == 0) return nullptr;
    slot.ctx_id = id;
    slot.ptr = p;
    return p;
}

}  // namespace gls

#endif  // GLS_SCRATCH_SLOT_H
