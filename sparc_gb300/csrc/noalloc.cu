// No-allocation variant of the spectral -> physical plane transform.
//
// Who needs it: callers that must not call cudaMalloc while they run.  A
// host application that has already handed the whole of HBM to its own pool
// (for example a driver that keeps hundreds of wavefield snapshots resident)
// gets out-of-memory from any further cudaMalloc; and cudaMalloc/cudaFree can
// synchronise the device, which stalls the other solves running on other
// streams while an output thread converts seismogram planes.  Such callers
// pass their own device input and output buffers to this entry point, and the
// only extra memory it uses is the fixed array below.
//
// The scratch is the column-pass intermediate of the inverse transform
// (cols_fft writes it, rows_c2r reads it).  It lives in one file-scope
// __device__ array of SPARC_NOALLOC_SCRATCH_BYTES that every GPU which loads
// this library holds until the process exits.  All calls share it:
//   - nothing in it has to start at zero: the column pass writes every
//     element the row pass reads, so the previous call's contents are never
//     used;
//   - calls whose work overlaps on the GPU (two streams, or two host threads)
//     race on the array and corrupt each other's output.  Serialise them, e.g.
//     by issuing them on one stream.
#include <mutex>
#include <string>
#include "internal.cuh"
#include "../../include/sparc_gpu.h"

static __device__ __align__(256) unsigned char g_noalloc_scratch[SPARC_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_mu;
constexpr int kMaxDevices = 256;
void* g_addr[kMaxDevices];
bool g_ready[kMaxDevices];

// Device address of the scratch array for the current device.  Host code may
// not use g_noalloc_scratch itself as a device pointer (on the host it names a
// shadow variable), so the address is looked up once per device, with that
// device current, and cached.
int scratch_address(void** out, std::string& why) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        why = std::string("cudaGetDevice failed: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return SPARC_ECUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        why = "device index " + std::to_string(dev) + " is outside the no-allocation address table (devices 0.." +
              std::to_string(kMaxDevices - 1) + ")";
        return SPARC_EINVAL;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_ready[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress((void**)&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || ptr == nullptr) {
            why = std::string("cudaGetSymbolAddress of the no-allocation scratch failed: ") + cudaGetErrorString(e);
            cudaGetLastError();
            return SPARC_ECUDA;
        }
        g_addr[dev] = ptr;
        g_ready[dev] = true;
    }
    *out = g_addr[dev];
    return SPARC_OK;
}
}  // namespace

extern "C" int sparc_gpu_spec_to_phys_noalloc(sparc_ctx* ctx, const void* spec, void* phys, int nplanes,
                                              void* stream) {
    if (!ctx) return SPARC_EINVAL;
    SparcXformInfo X;
    sparc_internal_xform_info(ctx, &X);
    if (!spec || !phys || nplanes < 1) {
        sparc_internal_set_error(ctx, "spec_to_phys_noalloc: null buffer or nplanes < 1");
        return SPARC_EINVAL;
    }
    const size_t cbytes = X.f32 ? sizeof(float2) : sizeof(double2);
    const size_t need = (X.ny > 1) ? (size_t)nplanes * (size_t)X.M * cbytes : 0;
    if (need > (size_t)SPARC_NOALLOC_SCRATCH_BYTES) {
        size_t per = (size_t)X.M * cbytes;
        sparc_internal_set_error(
            ctx, "spec_to_phys_noalloc: " + std::to_string(nplanes) + " planes need " + std::to_string(need) +
                     " bytes of scratch; the no-allocation limit is " +
                     std::to_string((size_t)SPARC_NOALLOC_SCRATCH_BYTES) + " bytes, i.e. at most " +
                     std::to_string((size_t)SPARC_NOALLOC_SCRATCH_BYTES / per) + " planes of this grid per call");
        return SPARC_EINVAL;
    }
    void* scratch = nullptr;
    std::string why;
    int rc = scratch_address(&scratch, why);
    if (rc != SPARC_OK) {
        sparc_internal_set_error(ctx, why);
        return rc;
    }
    cudaStream_t s = stream ? (cudaStream_t)stream : X.stream;
    if (X.f32)
        fft_spec_to_phys<float>((const float2*)spec, (float*)phys, (float2*)scratch, X.nx, X.ny, nplanes, X.tw_x,
                                X.tw_y, s);
    else
        fft_spec_to_phys<double>((const double2*)spec, (double*)phys, (double2*)scratch, X.nx, X.ny, nplanes, X.tw_x,
                                 X.tw_y, s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        sparc_internal_set_error(ctx, std::string("spec_to_phys_noalloc launch: ") + cudaGetErrorString(e));
        return SPARC_ECUDA;
    }
    sparc_internal_count_launches(ctx, X.ny > 1 ? 2 : 1);
    return SPARC_OK;
}
