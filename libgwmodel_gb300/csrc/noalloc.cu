// noalloc.cu -- a criterion entry point that never allocates device memory.
//
// Some callers cannot let a library call cudaMalloc: an application that owns
// all device memory through its own pool or budget, or a process that must not
// allocate after start-up (real-time serving, where cudaMalloc and cudaFree
// synchronise the device and stall every stream).
// gwgpu_criterion_noalloc serves them: the caller passes every input and
// output as device pointers, and the only scratch -- per-row hat diagonals and
// residuals and the per-block partial sums of the warp-per-location solve --
// lives in one file-scope __device__ array of fixed size (about 1.2 MB), which
// every GPU that loads the library holds until the process exits.
//
// The array is shared by every call on a device and keeps the previous call's
// contents; nothing in it has to start at zero (each launch overwrites the
// entries it later reads).  Calls whose work overlaps on the GPU -- two
// streams, or two host threads -- race on it, so callers serialise them.
//
// The first call on a device looks the array's device address up with
// cudaGetSymbolAddress (once per device, with that device current); make
// that first call before any stream capture begins.
#include <cfloat>
#include <cmath>
#include <cstddef>
#include <mutex>

#include "../../include/gwgpu.h"
#include "gw_kernels.h"

namespace gwgpu {
void set_last_error(const char* msg);
}

namespace {

constexpr int kNoAllocMaxRows = 65536;    // largest n accepted
constexpr int kNoAllocMaxBlocks = gwgpu::kSolveMaxBlocks;  // the largest grid launch_solve uses
constexpr int kNoAllocMaxDevices = 64;

struct NoAllocScratch {
    double sii[kNoAllocMaxRows];
    double resid[kNoAllocMaxRows];
    double partials[kNoAllocMaxBlocks * 4];
};
static_assert(sizeof(NoAllocScratch::partials) >= sizeof(double) * 4 * gwgpu::kSolveMaxBlocks,
              "the partial sums must hold every block launch_solve can use");

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

std::mutex g_noalloc_mu;
void* g_noalloc_addr[kNoAllocMaxDevices] = {};

// sums[4] = AICc (GWRBase::AICc, GWRBase.h:90-94) or CV from the reduced sums,
// DBL_MAX when a local system failed or the value is not finite.
__global__ void k_noalloc_value(int n, int criterion, double* sums)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double v;
    if (sums[3] > 0.0) {
        v = DBL_MAX;
    } else if (criterion == GWGPU_CV) {
        v = sums[1];
    } else {
        const double nn = (double)n, rss = sums[1], trS = sums[0];
        v = nn * log(rss / nn) + nn * log(2 * M_PI) + nn * ((nn + trS) / (nn - 2 - trS));
    }
    sums[4] = isfinite(v) ? v : DBL_MAX;
}

int fail(int code, const char* msg)
{
    gwgpu::set_last_error(msg);
    return code;
}

}  // namespace

extern "C" int gwgpu_criterion_noalloc(int n, int p, int criterion, int kernel, double bandwidth, const double* G,
                                       const double* X, const double* y, const double* thr, double* beta,
                                       double* sums, void* stream)
{
    if (n < 3 || n > kNoAllocMaxRows)
        return fail(GWGPU_ERR_INVALID, "gwgpu_criterion_noalloc: n must be in [3, 65536] (fixed scratch size)");
    if (p < 1 || p > gwgpu::kMaxP) return fail(GWGPU_ERR_INVALID, "gwgpu_criterion_noalloc: p must be in [1, 32]");
    if (criterion != GWGPU_AIC && criterion != GWGPU_CV)
        return fail(GWGPU_ERR_INVALID, "gwgpu_criterion_noalloc: unknown criterion");
    if (kernel < 0 || kernel > 4) return fail(GWGPU_ERR_INVALID, "gwgpu_criterion_noalloc: unknown kernel");
    if (!G || !X || !y || !beta || !sums) return fail(GWGPU_ERR_INVALID, "gwgpu_criterion_noalloc: null pointer");
    int dev = 0;
    cudaError_t rc = cudaGetDevice(&dev);
    if (rc != cudaSuccess) return fail(GWGPU_ERR_CUDA, cudaGetErrorString(rc));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(GWGPU_ERR_INVALID, "gwgpu_criterion_noalloc: device id");
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_addr[dev]) {
            rc = cudaGetSymbolAddress(&g_noalloc_addr[dev], g_noalloc_scratch);
            if (rc != cudaSuccess) {
                g_noalloc_addr[dev] = nullptr;
                return fail(GWGPU_ERR_CUDA, cudaGetErrorString(rc));
            }
        }
        base = g_noalloc_addr[dev];
    }
    unsigned char* b = static_cast<unsigned char*>(base);
    gwgpu::SolveArgs a{};
    a.n = n;
    a.p = p;
    a.mode = criterion == GWGPU_CV ? gwgpu::kSolveCV : gwgpu::kSolveAIC;
    a.kernel = kernel;
    a.G = G;
    a.ldg = p * (p + 1) / 2 + p;
    a.X = X;
    a.y = y;
    a.thr = thr;
    a.bw = bandwidth;
    a.beta = beta;
    a.sii = reinterpret_cast<double*>(b + offsetof(NoAllocScratch, sii));
    a.resid = reinterpret_cast<double*>(b + offsetof(NoAllocScratch, resid));
    a.partials = reinterpret_cast<double*>(b + offsetof(NoAllocScratch, partials));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    int nblocks = 0;
    rc = gwgpu::launch_solve(a, &nblocks, s);  // at most kSolveMaxBlocks blocks (static_assert above)
    if (rc != cudaSuccess) return fail(GWGPU_ERR_CUDA, cudaGetErrorString(rc));
    rc = gwgpu::launch_reduce_partials(a.partials, nblocks, sums, s);
    if (rc != cudaSuccess) return fail(GWGPU_ERR_CUDA, cudaGetErrorString(rc));
    k_noalloc_value<<<1, 32, 0, s>>>(n, criterion, sums);
    rc = cudaGetLastError();
    if (rc != cudaSuccess) return fail(GWGPU_ERR_CUDA, cudaGetErrorString(rc));
    return GWGPU_OK;
}
