// ref_stubs.cpp -- link stubs for building the reference's own host triplet->BSR routine
// (warp/native/sparse.cpp, compiled unmodified from the Warp source tree) into a small
// shared library under oracle/_ref/.  Test infrastructure only.
//
// The reference file references the APIC capture recorder and the host allocator.  Recording
// is never active here (wp_apic_get_recording_state() returns nullptr, so sparse.cpp takes its
// normal execution path); the allocator maps to malloc/free.  The remaining recorder entry
// points are unreachable and abort if ever called.
#include <cstdint>
#include <cstdlib>

#include "warp.h"
#include "apic.h"
#include "apic_internal.h"

extern "C" {
WP_API void* wp_alloc_host(size_t s, const char*) { return std::malloc(s); }
WP_API void wp_free_host(void* ptr) { std::free(ptr); }
WP_API APICState* wp_apic_get_recording_state() { return nullptr; }
}

APICAddress apic_resolve_host_ptr(APICState*, uint64_t, uint64_t) { std::abort(); }

void apic_record_bsr_transpose(APICState*, int, int, int, int, uint64_t, int, uint64_t, int, uint64_t, int, uint64_t,
                               int, uint64_t, int, uint64_t, int, uint64_t, int, uint64_t, const int32_t*, int)
{
    std::abort();
}

void apic_record_bsr_from_triplets(APICState*, int, int, int, int, int, uint64_t, uint8_t, int, uint64_t, int,
                                   uint64_t, int, uint64_t, int, uint64_t, int, uint64_t, int, uint64_t, int, uint64_t,
                                   int, uint64_t, int, uint64_t, int, uint64_t)
{
    std::abort();
}
