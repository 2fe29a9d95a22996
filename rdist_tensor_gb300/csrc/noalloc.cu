// Allocation-free variant of exafac_pinv_square.
//
// Some callers cannot allocate device memory or size a workspace in advance:
// code that runs under a memory pool owned by another framework, code in a
// latency-critical loop where cudaMalloc (which can synchronise the device)
// is not allowed, or code embedded where a fixed memory budget was set at
// start-up.  For them this entry point takes only its input and output: the
// eigenvector scratch of the Jacobi fallback lives in the file-scope array
// below, sized for the largest supported rank (R <= 128).
//
// The array is a module global: every GPU that loads this library holds its
// 128 KiB until the process exits, and all calls on a device share it.  The
// kernel writes every scratch element it reads (the Jacobi iteration starts
// from the identity), so nothing needs clearing between calls; calls whose
// kernels overlap on the GPU (different streams, no ordering) race on it.
//
// Host code cannot pass `g_pinv_scratch` itself to a kernel: in host code the
// name denotes a host-side stand-in, not a device address.  The first call on
// each device looks up the device address with cudaGetSymbolAddress (with
// that device current) and caches it; make that first call before any stream
// capture starts.  The cache lasts as long as the process: a device reset
// (cudaDeviceReset, or a reset of the primary context) reloads the module at
// another address, so the entry point must not be used on a device reset
// after its first call there.
#include <mutex>

#include "dense.cuh"

namespace exafac {

constexpr int kStaticMaxRank = 128;
constexpr int kStaticScratchDoubles = kStaticMaxRank * kStaticMaxRank;  // R_even^2, R_even <= 128

static __device__ __align__(256) double g_pinv_scratch[kStaticScratchDoubles];

static std::mutex g_scratch_mu;
static double* g_scratch_addr[64] = {nullptr};

static int static_scratch(double** out) {
    int dev = 0;
    EXAFAC_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("exafac_pinv_square_static: device ordinal out of range");
        return EXAFAC_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (g_scratch_addr[dev] == nullptr) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_pinv_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_error(std::string("exafac_pinv_square_static: cudaGetSymbolAddress failed: ") +
                      cudaGetErrorString(e));
            return EXAFAC_ERR_CUDA;
        }
        g_scratch_addr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_addr[dev];
    return EXAFAC_OK;
}

}  // namespace exafac

using namespace exafac;

extern "C" int exafac_pinv_square_static(int32_t R, const double* A, double* out, double tol, void* stream) {
    EXAFAC_ARG(R >= 1, "exafac_pinv_square_static: R must be >= 1");
    EXAFAC_ARG(R <= kStaticMaxRank,
               "exafac_pinv_square_static: R exceeds 128, the rank the static scratch is sized for");
    EXAFAC_ARG(A && out, "exafac_pinv_square_static: null pointer");
    double* scratch = nullptr;
    EXAFAC_TRY(static_scratch(&scratch));
    return launch_pinv(R, A, out, tol, scratch, (cudaStream_t)stream);
}
