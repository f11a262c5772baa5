// Internal definitions of libeqc (GB300 / sm_103a implementation of the eqcycle hot path).
#pragma once
#include <cuda_runtime.h>
#include <cuda.h>
#include <cstdint>
#include <unordered_map>
#include <cstdio>
#include <string>
#include <vector>
#include <stdexcept>
#include "../../include/eqc.h"

namespace eqc {

// ---- errors -----------------------------------------------------------------------
struct Error : std::runtime_error {
    eqc_status code;
    Error(eqc_status c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define EQC_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            throw ::eqc::Error(EQC_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_) + \
                                               " (" + __FILE__ + ":" + std::to_string(__LINE__) + ")"); \
    } while (0)

#define EQC_CHECK_LAUNCH() EQC_CUDA(cudaGetLastError())

// First statement of every kernel: wait until the grids this launch depends on have completed
// and their memory is visible.  A no-op for an ordinary launch; in the step graphs, edges
// between consecutive kernels are programmatic (make_programmatic), so a kernel's CTAs are
// scheduled while its predecessor is still running and start work as soon as it finishes.
#if defined(__CUDA_ARCH__)
#define EQC_GRID_WAIT() asm volatile("griddepcontrol.wait;" ::: "memory")
#else
#define EQC_GRID_WAIT() do {} while (0)
#endif

// ---- device buffer ----------------------------------------------------------------
template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DBuf() { release(); }
    void alloc(size_t count) {
        release();
        if (count == 0) return;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            throw Error(EQC_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        n = count;
        // cudaMemset runs on the legacy default stream, which does not order with the
        // handle's non-blocking stream: finish it before any upload can be enqueued.
        EQC_CUDA(cudaMemset(p, 0, count * sizeof(T)));
        EQC_CUDA(cudaDeviceSynchronize());
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void upload(const T* h, size_t count, cudaStream_t s) {
        if (count) EQC_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void upload(const std::vector<T>& h, cudaStream_t s) {
        if (n < h.size()) alloc(h.size());
        upload(h.data(), h.size(), s);
    }
    void download(T* h, size_t count, cudaStream_t s) const {
        if (count) EQC_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    void zero(cudaStream_t s) {
        if (n) EQC_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
};

// ---- node layout ------------------------------------------------------------------
// Lexicographic grid of GLL nodes: ix along depth (fast), iy fault-normal.  Node
// (ix, iy) lives at iy*ld + ix.  The fault is row iy = 0 and ix grows from the bottom
// of the fault (x = -LX) to the free surface, the same order as iFlt.
struct Layout {
    int NelX, NelY;
    int nx, ny;   // 4*NelX+1, 4*NelY+1
    int ld;       // row pitch in elements
    __host__ __device__ int64_t size() const { return (int64_t)ld * ny; }
    __host__ __device__ int64_t interior_begin() const { return ld; }   // first entry of row 1
};

// TMA tensor maps of the stiffness apply: one per node vector (keyed by its address) and
// one for the padded element data, per precision.
struct TmaCache {
    bool ok = false, walk_ok = false;
    std::unordered_map<const void*, CUtensorMap> u32, u64, u32walk;
    CUtensorMap w32, w64, w32walk;
};

// W padded to a 16-byte multiple per element, so element tiles are TMA-addressable.
template <class T> struct WPad;
template <> struct WPad<float> { static constexpr int v = 28; };
template <> struct WPad<double> { static constexpr int v = 26; };

// Stiffness apply parameters (element data in the reference's [i,j,e] layout,
// element e = ey*NelX + ex, src/MaterialProperties.jl:9).
template <class T>
struct ApplyArgs {
    const T* W;       // [25*Nel]
    T c1, c2;         // coefint1, coefint2 (par.jl:35-36)
    Layout L;
    const T* Wp;      // [WPad*Nel] padded copy for TMA (may be null)
    int* err;         // device flag set when a bounded wait gives up (may be null)
    TmaCache* tma;    // host-side tensor-map cache (may be null)
    int variant;      // see eqc_options.apply_variant
    int wait_polls;   // poll bound of a TMA kernel's first tile wait (the later waits and the
                      // drain after a give-up keep MBAR_SPIN_LIMIT); lowered only to test the
                      // give-up path (eqc_set_scalar "tma_wait_polls")
    const int* gate = nullptr;   // when set, the launch does nothing unless *gate (written by a
    int gate_val = 0;            // preceding kernel) equals gate_val
};

// Bound, in polls of mbarrier.try_wait, of every wait of the TMA-fed stiffness applies.
constexpr int MBAR_SPIN_LIMIT = 1 << 22;

// Error text for entry points without a handle (returned by eqc_last_error(NULL)).
void set_thread_error(const std::string& msg);

// Kernel counters (what the library launched).  While a graph is being captured the
// count goes to a capture tally instead; graph launches add what they execute.
extern int64_t g_launches;
extern thread_local int64_t* g_count_target;
inline void count_launch(int n = 1) { *(g_count_target ? g_count_target : &g_launches) += n; }

}  // namespace eqc
