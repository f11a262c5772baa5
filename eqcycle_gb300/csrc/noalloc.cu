// eqc_dtevol_noalloc: the adaptive time step of dtevol! computed over device arrays the
// caller already owns, with no device allocation of any kind.
//
// Why: some callers cannot allocate device memory -- a host code that hands the solver a
// fixed device arena, a caller running under a memory-budgeted allocator that forbids
// cudaMalloc from libraries, or one that needs the call to be usable where allocation
// would synchronise the device.  eqc_dtevol needs a handle, and creating a handle
// allocates.  This entry point needs neither: its reduction scratch (per-CTA partial minima
// and a completion counter) lives in a file-scope __device__ array of fixed size that every
// GPU loading this library holds until the process exits.
//
// Limits and sharing: at most EQC_NOALLOC_MAX_NODES fault nodes per call.  All calls share
// the one scratch array, which keeps the last call's contents; the completion counter is
// cleared (cudaMemsetAsync, no allocation) at the start of every call.  Calls that overlap
// on the GPU (concurrent streams, or several host threads) race on that scratch and must be
// serialised by the caller.  On the first call on a device the library looks up the
// device address of the scratch array (cudaGetSymbolAddress, with that device current)
// and caches it; make that first call before any stream capture.
#include "common.h"
#include <mutex>

namespace eqc {

constexpr int NA_THREADS = 256;
constexpr int NA_MAX_BLOCKS = 256;

struct DtevolScratch {
    double part[NA_MAX_BLOCKS];   // per-CTA minimum of XiLf/|V|
    unsigned int count;           // CTAs finished (last one reduces and clears it)
};

static __device__ __align__(256) DtevolScratch g_dtevol_scratch;

__global__ void __launch_bounds__(NA_THREADS) k_dtevol_noalloc(const double* __restrict__ Vf,
                                                                const double* __restrict__ XiLf, int64_t n,
                                                                int64_t first, double dt, double dtmin, int isolver,
                                                                DtevolScratch* S, double* out) {
    EQC_GRID_WAIT();
    __shared__ double smin[NA_THREADS / 32];
    __shared__ bool last;
    const double dtmax = 50.0 * 24 * 60 * 60;  // src/dtevol.jl:7
    double m = dtmax;
    for (int64_t i = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double sr = fabs(Vf[i]);
        if (sr * dtmax > XiLf[i]) m = fmin(m, XiLf[i] / sr);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = dtmax;
        for (int w = 0; w < NA_THREADS / 32; ++w) b = fmin(b, smin[w]);
        S->part[blockIdx.x] = b;
        __threadfence();
        last = (atomicAdd(&S->count, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    __threadfence();
    double dtnx = dtmax;
    for (unsigned k = 0; k < gridDim.x; ++k) dtnx = fmin(dtnx, __ldcg(&S->part[k]));
    double r;
    if (isolver == 1) {
        if (dtmin > dtnx) dtnx = dtmin;
        if (dtnx > 1.2 * dt) dtnx = 1.2 * dt;
        r = dtnx;
    } else {
        r = dtmin;
    }
    *out = r;
    S->count = 0u;
}

static std::mutex g_na_mutex;
static DtevolScratch* g_na_addr[64] = {nullptr};

}  // namespace eqc

using namespace eqc;

extern "C" eqc_status eqc_dtevol_noalloc(const double* Vf, const double* XiLf, int64_t n, int64_t NFBC, double dt,
                                         double dtmin, int32_t isolver, double* dt_out, void* stream) {
    if (!Vf || !XiLf || !dt_out || n < 1 || NFBC < 1 || NFBC > n + 1 || (isolver != 1 && isolver != 2)) {
        eqc::set_thread_error("eqc_dtevol_noalloc: invalid argument");
        return EQC_E_ARG;
    }
    if (n > EQC_NOALLOC_MAX_NODES) {
        eqc::set_thread_error("eqc_dtevol_noalloc: more fault nodes than EQC_NOALLOC_MAX_NODES");
        return EQC_E_ARG;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        eqc::set_thread_error("eqc_dtevol_noalloc: no current CUDA device");
        return EQC_E_NOGPU;
    }
    DtevolScratch* S;
    {
        std::lock_guard<std::mutex> lk(g_na_mutex);
        if (!g_na_addr[dev]) {
            void* p = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&p, g_dtevol_scratch);
            if (e != cudaSuccess || !p) {
                eqc::set_thread_error((std::string("eqc_dtevol_noalloc: cudaGetSymbolAddress: ") +
                                      cudaGetErrorString(e)).c_str());
                return EQC_E_CUDA;
            }
            g_na_addr[dev] = static_cast<DtevolScratch*>(p);
        }
        S = g_na_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemsetAsync(&S->count, 0, sizeof(unsigned int), s) != cudaSuccess) {
        eqc::set_thread_error("eqc_dtevol_noalloc: clearing the scratch counter failed");
        return EQC_E_CUDA;
    }
    const int64_t work = n - (NFBC - 1);
    int blocks = (int)std::min<int64_t>((work + NA_THREADS - 1) / NA_THREADS, NA_MAX_BLOCKS);
    if (blocks < 1) blocks = 1;
    k_dtevol_noalloc<<<blocks, NA_THREADS, 0, s>>>(Vf, XiLf, n, NFBC - 1, dt, dtmin, isolver, S, dt_out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        eqc::set_thread_error((std::string("eqc_dtevol_noalloc: launch: ") + cudaGetErrorString(e)).c_str());
        return EQC_E_CUDA;
    }
    count_launch();
    return EQC_OK;
}
