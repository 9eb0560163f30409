// bm_particle_contacts_static: the pair-contact pass of bm_particle_contacts
// with the bucket-scan workspace of its pair-list rebuild taken from a fixed
// static device array, so the call allocates nothing and needs no workspace
// from its caller beyond the buffers bound at bm_solver_create.
//
// Who needs it: a host that drives the contact pass from its own per-frame
// loop with a device-memory budget fixed at start-up (for example a rigid-body
// engine's contact callback), where an allocation would stall the frame or
// fail outright once the budget is taken.  The kernels, their order and
// their results are those of bm_particle_contacts.
#include <mutex>

#include "bm_device.cuh"
#include "bm_internal.h"

// Scan partials: one int per 1024 buckets of the pair-list hash table.
// 16384 partials (64 KiB) cover tables of up to 16,777,216 buckets, i.e.
// solvers of up to 8,388,608 particles at two buckets per particle.
// Nothing here has to start at zero: each rebuild writes every partial it
// reads earlier in the same call.
static __device__ __align__(256) int32_t g_scan_partials[BM_STATIC_SCAN_PARTIALS];

namespace {

constexpr int64_t kStaticPartials = BM_STATIC_SCAN_PARTIALS;
constexpr int kMaxDevices = 64;
std::mutex g_mutex;
int32_t* g_partials[kMaxDevices] = {};

// Device address of g_scan_partials on the current device.  The first call on
// each device makes the one runtime query (cudaGetSymbolAddress, which may
// load this library's device code on that device); later calls read the
// cached pointer.  The cache is never invalidated: it assumes the device's
// primary context lives as long as the process, so a cudaDeviceReset (after
// which the module may load at another address) ends this entry point's use
// in that process.
int static_partials(int32_t** out) {
    int device = -1;
    if (cudaGetDevice(&device) != cudaSuccess) return bm::check_cuda("particle_contacts_static: current device");
    if (device < 0 || device >= kMaxDevices)
        return bm::fail(BM_ERR_ARGUMENT, "particle_contacts_static: device ordinal beyond the 64 this library tracks");
    std::lock_guard<std::mutex> hold(g_mutex);
    if (!g_partials[device]) {
        void* address = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&address, g_scan_partials);
        if (rc != cudaSuccess || !address) {
            cudaGetLastError();
            return bm::fail(BM_ERR_CUDA, "particle_contacts_static: cudaGetSymbolAddress of the static scan partials failed");
        }
        g_partials[device] = static_cast<int32_t*>(address);
    }
    *out = g_partials[device];
    return BM_OK;
}

}  // namespace

extern "C" {

int bm_particle_contacts_static(bm_solver* s, void* stream) {
    if (!s) return bm::fail(BM_ERR_ARGUMENT, "null solver");
    const int64_t tiles = ((int64_t)s->P.bucket_mask + 1 + 1023) / 1024;
    if (tiles > kStaticPartials)
        return bm::fail(BM_ERR_ARGUMENT,
                        "particle_contacts_static: the pair-list table has more than 16,777,216 buckets "
                        "(16384 static scan partials); use bm_particle_contacts");
    int32_t* partials = nullptr;
    const int rc = static_partials(&partials);
    if (rc != BM_OK) return rc;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    bm::launch_prologue(s, 0, st);
    bm::launch_pairs_using(s, partials, st);
    return bm::check_cuda("particle_contacts_static");
}

}  // extern "C"
