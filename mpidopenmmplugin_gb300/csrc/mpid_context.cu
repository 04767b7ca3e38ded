// Host side of the GB300 MPIDForce evaluation: device buffers, cuFFT plans, the
// evaluation sequence and the induced-dipole solvers, behind the C ABI declared in
// include/mpid_gb300.h.  Replaces the reference's CUDA platform kernel
// (platforms/cuda/src/MPIDCudaKernels.cpp:711-1054).
#include <cuda_runtime.h>
#include <cufft.h>
#include <cub/device/device_radix_sort.cuh>
#include <cuda/std/tuple>
#include <cuda/std/utility>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <set>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "mpid_gb300.h"
#include "mpid_kernels.cuh"
#include "pme_host.h"
#include "radial_tables.h"

// ---------------------------------------------------------------------------
// Static scratch of the allocation-free evaluation (mpid_evaluate_device_noalloc).
// Some callers may not allocate device memory at the moment they evaluate: integrators
// that reserve a fixed device-memory budget up front and must stay inside it, or hosts
// whose own allocator owns the device memory (a caching allocator, a plugin host that
// forbids foreign cudaMalloc calls).  The ordinary evaluation allocates only when its
// neighbour lists outgrow their capacity; the allocation-free variant keeps the
// per-atom neighbour lists and the pair kernel's per-task energy partials in this fixed
// array instead and fails with MPID_ERR_INVALID rather than grow.  8 MiB: 1,835,008 list entries (npad x
// neighbours per atom, e.g. about 5,000 water atoms at a 0.9 nm cutoff) and 131,072
// FP64 task energies.  The array is one per device and per process, so calls must not
// overlap in time on a device (from any context, thread or stream): overlapping calls
// race on it.
namespace mpid {
constexpr size_t kNoAllocListEntries = 1835008;
constexpr size_t kNoAllocTasks = 131072;
constexpr size_t kNoAllocBytes = kNoAllocListEntries * 4 + kNoAllocTasks * 8;
constexpr int kNoAllocMaxDevices = 64;
}  // namespace mpid
static __device__ __align__(256) unsigned char g_noallocScratch[mpid::kNoAllocBytes];

namespace mpid {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CUDA_CHECK(x)                                                                              \
    do {                                                                                           \
        cudaError_t e_ = (x);                                                                      \
        if (e_ != cudaSuccess)                                                                     \
            throw Error(MPID_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));           \
    } while (0)
#define CUFFT_CHECK(x)                                                                             \
    do {                                                                                           \
        cufftResult r_ = (x);                                                                      \
        if (r_ != CUFFT_SUCCESS) throw Error(MPID_ERR_CUDA, std::string(#x) + " failed, code " + std::to_string((int) r_)); \
    } while (0)

static inline int nblk(long long n, int b) { return (int) ((n + b - 1) / b); }

// Makes `device` current for one C-ABI call and gives the caller's current device back
// at its end, so that a host thread driving several GPUs keeps its own choice.
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int device) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        CUDA_CHECK(cudaSetDevice(device));
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
};

// Kernel launches made by this thread (every launch of the library goes through
// launch<F>(); evaluations report their own count).
static thread_local long long t_launches = 0;

// ---------------------------------------------------------------------------
// Launch wrappers of the kernel bodies (MPID_KERNEL void F(KGrid<MT, MB>, P...)).
//  - k_one<F>: one launch of F, its parameters in the launch, the hardware block index.
//  - k_boxes<F>: one launch of F for many boxes (independent systems) at once.  The
//    launch's blocks are the concatenation of every box's blocks; a block finds its box
//    by a binary search over the boxes' first blocks and runs F with that box's
//    parameters and its rank within the box.  The parameter sets of all boxes travel in
//    the launch's parameter space (__grid_constant__, read through the constant cache),
//    up to BoxParams::kBoxes boxes per launch.
// Three variants each: the body's launch bounds in full, the thread bound only, none.
template <class F> struct KernelTraits;
template <int MT, int MB, class... P>
struct KernelTraits<void (*)(KGrid<MT, MB>, P...)> {
    static constexpr int maxThreads = MT, minBlocks = MB;
    using Args = cuda::std::tuple<P...>;
    using Grid = KGrid<MT, MB>;
};
template <auto F> using KTraits = KernelTraits<decltype(F)>;

template <class Args>
struct BoxParams {
    // as many boxes as keep the launch parameters within 31,000 bytes (the limit is 32,764)
    static constexpr int kBoxes = (int) ((31000 - 16) / (sizeof(Args) + 4)) < 64 ? (int) ((31000 - 16) / (sizeof(Args) + 4)) : 64;
    int count;
    unsigned first[kBoxes + 1];  // first block of each box; first[count] = blocks of the launch
    Args args[kBoxes];
};

template <auto F, class Args, size_t... I>
__device__ __forceinline__ void run_box_body(const Args& a, typename KTraits<F>::Grid g, cuda::std::index_sequence<I...>) {
    F(g, cuda::std::get<I>(a)...);
}
template <auto F>
__device__ __forceinline__ void run_boxes(const BoxParams<typename KTraits<F>::Args>& bp) {
    using Args = typename KTraits<F>::Args;
    const unsigned b = blockIdx.x;
    int lo = 0, hi = bp.count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (bp.first[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    run_box_body<F>(bp.args[lo], typename KTraits<F>::Grid{b - bp.first[lo], bp.first[lo + 1] - bp.first[lo]},
                    cuda::std::make_index_sequence<cuda::std::tuple_size<Args>::value>{});
}

template <auto F, class... P>
__global__ void k_one(P... p) { F(typename KTraits<F>::Grid{blockIdx.x, gridDim.x}, p...); }
template <auto F, class... P>
__global__ void __launch_bounds__(KTraits<F>::maxThreads) k_one_t(P... p) {
    F(typename KTraits<F>::Grid{blockIdx.x, gridDim.x}, p...);
}
template <auto F, class... P>
__global__ void __launch_bounds__(KTraits<F>::maxThreads, KTraits<F>::minBlocks) k_one_tb(P... p) {
    F(typename KTraits<F>::Grid{blockIdx.x, gridDim.x}, p...);
}
template <auto F>
__global__ void k_boxes(const __grid_constant__ BoxParams<typename KTraits<F>::Args> bp) { run_boxes<F>(bp); }
template <auto F>
__global__ void __launch_bounds__(KTraits<F>::maxThreads) k_boxes_t(const __grid_constant__ BoxParams<typename KTraits<F>::Args> bp) {
    run_boxes<F>(bp);
}
template <auto F>
__global__ void __launch_bounds__(KTraits<F>::maxThreads, KTraits<F>::minBlocks)
    k_boxes_tb(const __grid_constant__ BoxParams<typename KTraits<F>::Args> bp) {
    run_boxes<F>(bp);
}

template <class T> static inline T implicit_arg(T v) { return v; }

template <auto F, class Args> struct Launcher;
template <auto F, class... P>
struct Launcher<F, cuda::std::tuple<P...>> {
    template <class... A>
    static void one(dim3 grid, dim3 block, size_t smem, cudaStream_t st, A&&... a) {
        if constexpr (KTraits<F>::maxThreads == 0)
            k_one<F, P...><<<grid, block, smem, st>>>(implicit_arg<P>(std::forward<A>(a))...);
        else if constexpr (KTraits<F>::minBlocks == 0)
            k_one_t<F, P...><<<grid, block, smem, st>>>(implicit_arg<P>(std::forward<A>(a))...);
        else
            k_one_tb<F, P...><<<grid, block, smem, st>>>(implicit_arg<P>(std::forward<A>(a))...);
    }
    template <class... A>
    static cuda::std::tuple<P...> pack(A&&... a) { return cuda::std::tuple<P...>(implicit_arg<P>(std::forward<A>(a))...); }
};

template <auto F>
static void launch_boxes_now(const BoxParams<typename KTraits<F>::Args>& bp, dim3 block, size_t smem, cudaStream_t st) {
    const dim3 grid(bp.first[bp.count]);
    if constexpr (KTraits<F>::maxThreads == 0)
        k_boxes<F><<<grid, block, smem, st>>>(bp);
    else if constexpr (KTraits<F>::minBlocks == 0)
        k_boxes_t<F><<<grid, block, smem, st>>>(bp);
    else
        k_boxes_tb<F><<<grid, block, smem, st>>>(bp);
}

// ---------------------------------------------------------------------------
// Recording of an evaluation's device work (fused multi-box evaluation): while a thread
// has a recorder, launch<F>() and the op_* helpers append operations to it instead of
// issuing them, each with the stream it was issued on; event records and waits are
// operations too, so that the recording keeps the evaluation's stream structure.
struct RecKernel {
    dim3 grid, block;
    size_t smem = 0;
    virtual ~RecKernel() = default;
    virtual const void* body() const = 0;  // one address per kernel body
    // one launch (or one per BoxParams::kBoxes boxes) of this body for all of `group`
    virtual void launch_group(const std::vector<const RecKernel*>& group, cudaStream_t st) const = 0;
};
template <auto F>
struct RecKernelOf : RecKernel {
    typename KTraits<F>::Args args;
    static const void* tag() {
        static const char t = 0;
        return &t;
    }
    const void* body() const override { return tag(); }
    void launch_group(const std::vector<const RecKernel*>& group, cudaStream_t st) const override {
        using BP = BoxParams<typename KTraits<F>::Args>;
        std::unique_ptr<BP> bp(new BP());
        for (size_t s = 0; s < group.size(); s += BP::kBoxes) {
            const size_t m = std::min<size_t>(BP::kBoxes, group.size() - s);
            bp->count = (int) m;
            unsigned total = 0;
            size_t smemMax = 0;
            for (size_t i = 0; i < m; ++i) {
                const auto* r = static_cast<const RecKernelOf<F>*>(group[s + i]);
                bp->first[i] = total;
                bp->args[i] = r->args;
                total += r->grid.x;
                smemMax = std::max(smemMax, r->smem);
            }
            bp->first[m] = total;
            launch_boxes_now<F>(*bp, block, smemMax, st);
            ++t_launches;
        }
    }
};

struct RecOp {
    enum Kind { KERNEL, FILL, COPY, FFT, EV_RECORD, EV_WAIT } kind;
    cudaStream_t stream = nullptr;               // the stream it was issued on
    cudaEvent_t event = nullptr;                 // EV_RECORD, EV_WAIT
    std::unique_ptr<RecKernel> k;                // KERNEL
    void* dst = nullptr;                         // FILL, COPY, FFT (output grid)
    const void* src = nullptr;                   // COPY, FFT (input grid)
    size_t bytes = 0;                            // FILL, COPY
    int value = 0;                               // FILL (byte value)
    int fftDims[3] = {0, 0, 0}, fftPrec = 0, fftForward = 0;  // FFT: grid, 4 or 8 byte reals, direction
};

struct OpRecorder {
    std::vector<RecOp> ops;
};
static thread_local OpRecorder* t_recorder = nullptr;

template <auto F, class... A>
static inline void launch(dim3 grid, dim3 block, size_t smem, cudaStream_t st, A&&... a) {
    using L = Launcher<F, typename KTraits<F>::Args>;
    if (t_recorder) {
        if (grid.y != 1 || grid.z != 1) throw std::logic_error("recorded launches must be one-dimensional");
        std::unique_ptr<RecKernelOf<F>> r(new RecKernelOf<F>());
        r->grid = grid;
        r->block = block;
        r->smem = smem;
        r->args = L::pack(std::forward<A>(a)...);
        RecOp op;
        op.kind = RecOp::KERNEL;
        op.stream = st;
        op.k = std::move(r);
        t_recorder->ops.push_back(std::move(op));
        return;
    }
    L::one(grid, block, smem, st, std::forward<A>(a)...);
    ++t_launches;
}
// cuFFT executions and cub sorts (library code launching its own kernels).
static thread_local long long t_library_calls = 0;

// Device work other than kernels, recorded like launches while a recorder is active.
static inline void op_memset(void* p, int value, size_t bytes, cudaStream_t st) {
    if (t_recorder) {
        RecOp op;
        op.kind = RecOp::FILL;
        op.stream = st;
        op.dst = p;
        op.value = value;
        op.bytes = bytes;
        t_recorder->ops.push_back(std::move(op));
        return;
    }
    CUDA_CHECK(cudaMemsetAsync(p, value, bytes, st));
}
// A device-to-device copy, or a device-to-host copy into pinned (device-mapped) memory.
static inline void op_copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st) {
    if (t_recorder) {
        RecOp op;
        op.kind = RecOp::COPY;
        op.stream = st;
        op.dst = dst;
        op.src = src;
        op.bytes = bytes;
        t_recorder->ops.push_back(std::move(op));
        return;
    }
    CUDA_CHECK(cudaMemcpyAsync(dst, src, bytes, kind, st));
}
static inline void op_record(cudaEvent_t ev, cudaStream_t st) {
    if (t_recorder) {
        RecOp op;
        op.kind = RecOp::EV_RECORD;
        op.stream = st;
        op.event = ev;
        t_recorder->ops.push_back(std::move(op));
        return;
    }
    CUDA_CHECK(cudaEventRecord(ev, st));
}
static inline void op_wait(cudaStream_t st, cudaEvent_t ev) {
    if (t_recorder) {
        RecOp op;
        op.kind = RecOp::EV_WAIT;
        op.stream = st;
        op.event = ev;
        t_recorder->ops.push_back(std::move(op));
        return;
    }
    CUDA_CHECK(cudaStreamWaitEvent(st, ev, 0));
}

// Device allocations made by any buffer so far: captured graphs key on it, so that no
// graph outlives a pointer it holds.
static std::atomic<unsigned long long> g_device_allocs{0};

// Simple owning device buffer.
template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    void alloc(size_t count) {
        if (count <= n && p) return;
        free();
        CUDA_CHECK(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
        n = count;
        ++g_device_allocs;
    }
    void free() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DBuf() { free(); }
};

// ---------------------------------------------------------------------------
template <typename real> struct FftTypes;
template <> struct FftTypes<float> {
    static constexpr cufftType fwd = CUFFT_R2C, inv = CUFFT_C2R;
    static void exec_fwd(cufftHandle h, float* in, float2* out) { ++t_library_calls; CUFFT_CHECK(cufftExecR2C(h, in, (cufftComplex*) out)); }
    static void exec_inv(cufftHandle h, float2* in, float* out) { ++t_library_calls; CUFFT_CHECK(cufftExecC2R(h, (cufftComplex*) in, out)); }
};
template <> struct FftTypes<double> {
    static constexpr cufftType fwd = CUFFT_D2Z, inv = CUFFT_Z2D;
    static void exec_fwd(cufftHandle h, double* in, double2* out) { ++t_library_calls; CUFFT_CHECK(cufftExecD2Z(h, in, (cufftDoubleComplex*) out)); }
    static void exec_inv(cufftHandle h, double2* in, double* out) { ++t_library_calls; CUFFT_CHECK(cufftExecZ2D(h, (cufftDoubleComplex*) in, out)); }
};

// One precision's PME machinery: B-spline tables of the sorted atoms, accumulation
// grid, real / half-complex FFT grids and plans.
template <typename real>
struct PmeStage {
    int order = 6, nx = 0, ny = 0, nz = 0;
    int sms = 1;  // multiprocessors of the device (grid-stride launch sizes)
    size_t G = 0, Gh = 0;
    DBuf<typename GridAcc<real>::type> acc;
    DBuf<real> rgrid;
    DBuf<typename Cplx<real>::type> cgrid;
    DBuf<real> theta;
    DBuf<int> igrid;
    cufftHandle fwd = 0, inv = 0;
    bool planned = false;

    void init(int ord, int gx, int gy, int gz, int npad, int numSMs) {
        order = ord;
        sms = numSMs;
        nx = gx; ny = gy; nz = gz;
        G = (size_t) nx * ny * nz;
        Gh = (size_t) nx * ny * (nz / 2 + 1);
        acc.alloc(G);
        rgrid.alloc(G);
        cgrid.alloc(Gh);
        theta.alloc((size_t) 3 * 5 * order * npad);
        igrid.alloc((size_t) 3 * npad);
        CUDA_CHECK(cudaMemset(acc.p, 0, G * sizeof(typename GridAcc<real>::type)));
        CUFFT_CHECK(cufftPlan3d(&fwd, nx, ny, nz, FftTypes<real>::fwd));
        CUFFT_CHECK(cufftPlan3d(&inv, nx, ny, nz, FftTypes<real>::inv));
        planned = true;
    }
    ~PmeStage() {
        if (planned) {
            cufftDestroy(fwd);
            cufftDestroy(inv);
        }
    }
    cudaStream_t planStream = nullptr;  // the stream the plans run on
    void set_stream(cudaStream_t s) {
        CUFFT_CHECK(cufftSetStream(fwd, s));
        CUFFT_CHECK(cufftSetStream(inv, s));
        planStream = s;
    }
    void bsplines(int n, int npad, const int* sorted, const double* wpos, const BoxDev& box, cudaStream_t st) {
        if (order == 5)
            launch<k_bsplines<real, 5>>(nblk(npad, 128), 128, 0, st, npad, n, sorted, wpos, box, theta.p, igrid.p);
        else
            launch<k_bsplines<real, 6>>(nblk(npad, 128), 128, 0, st, npad, n, sorted, wpos, box, theta.p, igrid.p);
    }
    template <int NCOMP>
    void spread(int n, int npad, const BoxDev& box, const real* mf, const int* skip, cudaStream_t st) {
        const long long threads = (long long) n * order * order;
        if (order == 5)
            launch<k_spread<real, 5, NCOMP>>(nblk(threads, 256), 256, 0, st, n, npad, box, mf, theta.p, igrid.p, acc.p, skip);
        else
            launch<k_spread<real, 6, NCOMP>>(nblk(threads, 256), 256, 0, st, n, npad, box, mf, theta.p, igrid.p, acc.p, skip);
        launch<k_grid_finish<real>>(std::min<long long>(nblk(G, 256), (long long) sms * 16), 256, 0, st, G, acc.p, rgrid.p,
               skip);
    }
    // Real-to-half-complex transform of rgrid into cgrid (forward) or back (inverse).
    void fft(bool forward) {
        if (t_recorder) {
            RecOp op;
            op.kind = RecOp::FFT;
            op.stream = planStream;
            op.src = forward ? (const void*) rgrid.p : (const void*) cgrid.p;
            op.dst = forward ? (void*) cgrid.p : (void*) rgrid.p;
            op.fftDims[0] = nx;
            op.fftDims[1] = ny;
            op.fftDims[2] = nz;
            op.fftPrec = (int) sizeof(real);
            op.fftForward = forward ? 1 : 0;
            t_recorder->ops.push_back(std::move(op));
            return;
        }
        if (forward)
            FftTypes<real>::exec_fwd(fwd, rgrid.p, cgrid.p);
        else
            FftTypes<real>::exec_inv(inv, cgrid.p, rgrid.p);
    }
    void convolve(const double* influence, const int* skip, cudaStream_t st) {
        fft(true);
        launch<k_convolve<real>>(std::min<long long>(nblk(Gh, 256), (long long) sms * 16), 256, 0, st, Gh, influence,
               cgrid.p, skip);
        fft(false);
    }
    template <int NTERM>
    void gather(int n, int npad, const BoxDev& box, real* phi, const int* skip, cudaStream_t st) {
        if (order == 5) {
            using G = GatherShape<real, 5, NTERM>;
            launch<k_gather<real, 5, NTERM>>(nblk(npad, G::atoms), G::threads, 0, st, n, npad, box, theta.p, igrid.p,
                   rgrid.p, phi, skip);
        } else {
            using G = GatherShape<real, 6, NTERM>;
            launch<k_gather<real, 6, NTERM>>(nblk(npad, G::atoms), G::threads, 0, st, n, npad, box, theta.p, igrid.p,
                   rgrid.p, phi, skip);
        }
    }
};

// Per-precision engine: sorted atom arrays, PME stage, field / force accumulators.
template <typename real>
struct Engine {
    int n = 0, npad = 0;
    DBuf<real> off, mom, alab, sroot;
    DBuf<typename Vec4<real>::type> prm;
    DBuf<int> orig, rank;
    DBuf<real> mf, mfd;                       // [20][npad], [4][npad]
    DBuf<real> phiP, phiD, phiT;              // [35][npad] each; phiT scratch
    DBuf<unsigned long long> fieldFx, gradFx;  // [3][npad], [6][npad]
    DBuf<real> Efix, muD, SE, mu, Etmp, Gtmp, sp;
    DBuf<real> zc;                             // preconditioned residual of the mutual CG
    DBuf<unsigned long long> precFx;           // [3][npad] near-field preconditioner field
    PmeStage<real> pme;
    bool usePme = false;

    AtomArrays<real> arrays() {
        AtomArrays<real> a;
        a.n = n; a.npad = npad;
        a.off = off.p; a.mom = mom.p; a.alab = alab.p; a.sroot = sroot.p;
        a.prm = prm.p; a.orig = orig.p; a.rank = rank.p;
        return a;
    }
    void init(int natoms, int pad, bool pme_, int order, const int* grid, int numSMs) {
        n = natoms;
        npad = pad;
        usePme = pme_;
        off.alloc(3 * (size_t) npad);
        mom.alloc(20 * (size_t) npad);
        alab.alloc(6 * (size_t) npad);
        sroot.alloc(6 * (size_t) npad);
        prm.alloc(npad);
        orig.alloc(npad);
        rank.alloc(std::max(n, 1));
        mf.alloc(20 * (size_t) npad);
        mfd.alloc(4 * (size_t) npad);
        phiP.alloc(35 * (size_t) npad);
        phiD.alloc(35 * (size_t) npad);
        phiT.alloc(35 * (size_t) npad);
        fieldFx.alloc(3 * (size_t) npad);
        gradFx.alloc(6 * (size_t) npad);
        Efix.alloc(3 * (size_t) npad);
        muD.alloc(3 * (size_t) npad);
        SE.alloc(3 * (size_t) npad);
        mu.alloc(3 * (size_t) npad);
        Etmp.alloc(3 * (size_t) npad);
        Gtmp.alloc(6 * (size_t) npad);
        sp.alloc(3 * (size_t) npad);
        zc.alloc(3 * (size_t) npad);
        precFx.alloc(3 * (size_t) npad);
        if (usePme) pme.init(order, grid[0], grid[1], grid[2], npad, numSMs);
    }
};

// Device time of the evaluation stages, from CUDA events on the launching stream.
enum Stage { ST_SETUP = 0, ST_FIXED_REAL, ST_PME, ST_DIPOLE_REAL, ST_FFT, ST_PAIR, ST_FINISH, ST_REFINE_REAL, ST_COUNT };

// Start/stop events of one timed stage.
struct TimedPair {
    int stage;
    cudaEvent_t a, b;
};

struct StageTimer {
    static constexpr int kMax = 4096;
    std::vector<cudaEvent_t> ev;
    std::vector<int> stage;
    int count = 0, open = -1;
    double ms[ST_COUNT] = {0};
    int launches[ST_COUNT] = {0};
    // Inside a stream capture the events are recorded as graph nodes
    // (cudaEventRecordExternal), drawn from the capturing graph's own pool, and the graph
    // keeps the pairs; each replay hands them back through `replayed`.  A graph replayed
    // more than once in an evaluation is timed by its last replay, once per replay.
    std::vector<cudaEvent_t>* capPool = nullptr;
    std::vector<TimedPair>* capPairs = nullptr;
    size_t capNext = 0;
    TimedPair capOpen{-1, nullptr, nullptr};
    std::vector<TimedPair> replayed;
    void init() {
        ev.resize(2 * kMax);
        stage.resize(kMax);
        for (auto& e : ev) CUDA_CHECK(cudaEventCreate(&e));
    }
    void destroy() {
        for (auto e : ev) cudaEventDestroy(e);
        ev.clear();
    }
    void reset() {
        count = 0;
        open = -1;
        replayed.clear();
        for (int s = 0; s < ST_COUNT; ++s) { ms[s] = 0; launches[s] = 0; }
    }
    bool off = false;  // set while a whole evaluation is captured for a batch (no stage events)
    void begin(int s, cudaStream_t st) {
        if (off) return;
        if (capPool) {
            if (capNext + 2 > capPool->size()) return;
            capOpen = {s, (*capPool)[capNext], (*capPool)[capNext + 1]};
            capNext += 2;
            CUDA_CHECK(cudaEventRecordWithFlags(capOpen.a, st, cudaEventRecordExternal));
            return;
        }
        if (count >= kMax || ev.empty()) return;
        stage[count] = s;
        CUDA_CHECK(cudaEventRecord(ev[2 * count], st));
        open = count;
    }
    void end(cudaStream_t st) {
        if (off) return;
        if (capPool) {
            if (capOpen.stage < 0) return;
            CUDA_CHECK(cudaEventRecordWithFlags(capOpen.b, st, cudaEventRecordExternal));
            capPairs->push_back(capOpen);
            capOpen.stage = -1;
            return;
        }
        if (open < 0) return;
        CUDA_CHECK(cudaEventRecord(ev[2 * open + 1], st));
        ++count;
        open = -1;
    }
    void add(int s, cudaEvent_t a, cudaEvent_t b) {
        float t = 0.f;
        if (cudaEventElapsedTime(&t, a, b) == cudaSuccess) {
            ms[s] += t;
            launches[s] += 1;
        }
    }
    // after the stream has been synchronised
    void collect() {
        for (int i = 0; i < count; ++i) add(stage[i], ev[2 * i], ev[2 * i + 1]);
        for (const TimedPair& p : replayed) add(p.stage, p.a, p.b);
        (void) cudaGetLastError();  // a pair that could not be timed leaves no error behind
    }
};

// ---------------------------------------------------------------------------
static std::atomic<unsigned long long> g_context_ids{0};

struct Context {
    mpid_settings set;
    int device = 0;
    unsigned long long id = ++g_context_ids;  // never reused: batch graphs key on it
    int numSMs = 1;  // multiprocessors of the device, read at creation (launch sizes)
    int n = 0, npad = 0, ntiles = 0;
    bool usePme = false, mixed = true;
    cudaStream_t stream = nullptr;
    // The context's own stream, used by the host-buffer calls so that contexts driven
    // from different host threads run concurrently.
    cudaStream_t hostStream = nullptr;
    // Side stream for the reciprocal-space (PME) chains, which run concurrently with the
    // real-space pair kernel on the main stream: fork_pme makes the side stream wait for
    // the main stream's work so far, join_pme makes the main stream wait for the side.
    cudaStream_t pmeStream = nullptr;
    cudaEvent_t evFork = nullptr, evJoin = nullptr;
    // The side streams the context owns; bind_streams points the working members at them,
    // or at the caller's stream under MPID_FLAG_SERIAL_STAGES.
    cudaStream_t pmeOwn = nullptr, refOwn = nullptr, refPmeOwn = nullptr;
    bool serialStages = false;
    void bind_streams() {
        pmeStream = serialStages ? stream : pmeOwn;
        refStream = serialStages ? stream : refOwn;
        refPmeStream = serialStages ? stream : refPmeOwn;
    }
    // The mixed Mutual solver's FP64 residual check runs on its own pair of streams,
    // concurrently with the force/energy phase that assumes it passes.
    cudaStream_t refStream = nullptr, refPmeStream = nullptr;
    cudaEvent_t evRefFork = nullptr, evRefJoin = nullptr, evRefStart = nullptr, evRefDone = nullptr;
    double* refHost = nullptr;  // pinned: squared residual sum of the pending check
    int refOuter = 0, refTotal = 0;
    void fork_pme() {
        op_record(evFork, stream);
        op_wait(pmeStream, evFork);
    }
    void join_pme() {
        op_record(evJoin, pmeStream);
        op_wait(stream, evJoin);
    }
    bool ownStream = false;

    // parameters (device, original order)
    DBuf<double> charge, dipole, quad, oct, thole, pol;
    DBuf<int> axis, az, ax, ay;
    std::vector<int> h_axis, h_az, h_ax, h_ay;
    bool haveParams = false;
    // covalent partners: symmetric CSR over original indices
    DBuf<int> covOff, covJ;
    DBuf<double> covS;
    // sort / tiles
    DBuf<unsigned> keys, keysAlt;
    DBuf<int> order, orderAlt;          // atom index of each sorted slot
    DBuf<char> cubTemp;
    size_t cubBytes = 0;
    DBuf<double> pos, wpos, center, half;
    DBuf<float4> centerF, halfF;        // the same in FP32 for the tile-pair tests
    // neighbour lists (tile lists, then per-atom lists; layouts in mpid_kernels.cuh)
    int tcap = 0, cap = 0, chunk = 32, nchunksL = 1, nchunksS = 0;
    DBuf<int> tileCount, tileJ, countL, countS, loL, loS, tmaxL, tmaxS, listMax;
    DBuf<float4> shF;
    DBuf<double> shD;
    DBuf<float2> shDF;
    // double-float inputs and Ewald tables of the mixed path's residual field
    DBuf<float2> offDF, muDF, tholeDF, dampDF;
    DBuf<float4> pack0, pack1;  // packed operands of the FP32 CG pair kernel
    CgRadial cgR{};             // its radial-function polynomials (cg_radial.h)
    DBuf<float> tabG, tabGc, tabH, tabHc;
    RadialTableHost tabGh, tabHh;
    DBuf<unsigned> list;
    int lastTiles = 0, lastMaxList = 0;
    long long listEntries = 0;
    bool growForbidden = false;  // set by the allocation-free entry point
    // The counts and segment sizes of the last list build describe lists that lived in
    // the allocation-free call's scratch, not in `list`: passes that read the lists
    // outside an evaluation must rebuild them first (every evaluation does).
    bool listsInScratch = false;
    // PME tables
    DBuf<double> modx, mody, modz, influence;
    double lastBox[9] = {0};
    // engines
    std::unique_ptr<Engine<float>> ef;
    std::unique_ptr<Engine<double>> ed;
    // FP64 engine of the gradient pass on the mixed path without a refinement engine
    // (Direct, Extrapolated); created on the first gradient request
    std::unique_ptr<Engine<double>> eg;
    // accumulators (sorted order)
    DBuf<unsigned long long> forceFx, torqueFx;
    DBuf<double> energyBlocks;          // per-block real-space energy
    DBuf<double> mom64, prm64;          // FP64 lab moments (sorted) and (thole, damp) by atom
    DBuf<int2> scaledPairs;             // covalently scaled pairs (i < j), original indices
    DBuf<double> scaledScale, scaledPartial;
    int nScaled = 0;
    DBuf<double> energyPartial, energyOut;
    DBuf<double> forcesOut;
    DBuf<double> masses, momentPartial, momentRed, gridPts, gridOut;  // system moments, potential
    DBuf<unsigned long long> gradFx;  // [20][npad] real-space parameter gradient
    DBuf<double> gradOut;             // [n][20]
    DBuf<int> atomTypes;              // per-atom parameter type (original order), mpid_set_atom_types
    std::vector<int> atomTypesHost;
    int ntypes = 0;
    DBuf<unsigned long long> polFx;   // [2][npad] screening sums W, Z of the polarisation gradient
    DBuf<double> gradPtMu, gradPtE, gradEfix;  // FP64 copies of the mixed path's OPT orders and fields
    DBuf<double> polOut;              // [n][4]
    // solver scratch
    DBuf<double> partial, red, sc;
    DBuf<int> iter, done;
    DBuf<unsigned> counters;  // last-block counters of the fused CG reductions
    DBuf<float> r32, p32, q32, x32, b32, s32;
    DBuf<double> r64, p64, q64, y64, b64, res64, Efix64, s64;
    DBuf<float> res32;
    // extrapolated
    DBuf<float> ptMuF, ptEF, ptGF;
    DBuf<double> ptMuD, ptED, ptGD;
    int* hostDone = nullptr;       // pinned: 256 iteration flags, then the solve's iteration count
    double* hostSc = nullptr;      // pinned: the solver scalars after a solve
    int* hostMax = nullptr;        // list maxima (pinned)
    cudaEvent_t evLists = nullptr;
    std::vector<cudaEvent_t> iterEvents;
    cudaEvent_t evStart = nullptr, evStop = nullptr;
    mpid_stats stats{};
    StageTimer timer;
    bool evaluated = false;
    bool gradPrepared = false;  // FP64 inputs of the gradient pass hold the last evaluation
    BoxDev box{};

    // Captured segments of the evaluation (MPID_FLAG_GRAPH_SOLVER); `key` holds every
    // value the launches bake in (graph_key), so a changed list shape, buffer or box
    // captures a new graph.
    struct SolverGraph {
        std::vector<long long> key;
        long long nodes = 0;  // kernel launches one replay stands for
        long long library = 0;
        unsigned long long used = 0;
        cudaGraphExec_t exec = nullptr;
        std::vector<cudaEvent_t> events;  // the stage timer's events inside the graph
        std::vector<TimedPair> pairs;
        void destroy() {
            if (exec) cudaGraphExecDestroy(exec);
            exec = nullptr;
            for (cudaEvent_t e : events) cudaEventDestroy(e);
            events.clear();
            pairs.clear();
        }
    };
    std::vector<SolverGraph> graphs;
    unsigned long long graphClock = 0;
    int predictedIters = 0;  // iterations of the last solve: the first replayed chunk's length

    ~Context() {
        for (auto& g : graphs) g.destroy();
        full.destroy();
        if (hostEparts) cudaFreeHost(hostEparts);
        timer.destroy();
        if (hostDone) cudaFreeHost(hostDone);
        if (hostSc) cudaFreeHost(hostSc);
        if (evFork) cudaEventDestroy(evFork);
        if (evJoin) cudaEventDestroy(evJoin);
        if (pmeOwn) cudaStreamDestroy(pmeOwn);
        if (hostMax) cudaFreeHost(hostMax);
        if (evLists) cudaEventDestroy(evLists);
        for (auto e : iterEvents) cudaEventDestroy(e);
        if (evStart) cudaEventDestroy(evStart);
        if (evStop) cudaEventDestroy(evStop);
        if (ownStream && stream) cudaStreamDestroy(stream);
        if (hostStream) cudaStreamDestroy(hostStream);
        if (refOwn) cudaStreamDestroy(refOwn);
        if (refPmeOwn) cudaStreamDestroy(refPmeOwn);
        for (cudaEvent_t e : {evRefFork, evRefJoin, evRefStart, evRefDone})
            if (e) cudaEventDestroy(e);
        if (refHost) cudaFreeHost(refHost);
    }

    // ----- set-up -----
    void create(const mpid_settings& s, int dev) {
        set = s;
        device = dev;
        n = s.num_atoms;
        if (n <= 0) throw Error(MPID_ERR_INVALID, "MPIDForce must have at least one particle");
        if (s.nonbonded_method != MPID_PME && s.nonbonded_method != MPID_NO_CUTOFF)
            throw Error(MPID_ERR_INVALID, "MPIDForce: Illegal value for nonbonded method");
        if (s.polarization_type < 0 || s.polarization_type > 2)
            throw Error(MPID_ERR_INVALID, "Polarization type not recognzied.");
        if (s.precision != MPID_PRECISION_MIXED && s.precision != MPID_PRECISION_DOUBLE)
            throw Error(MPID_ERR_INVALID, "unknown precision");
        usePme = s.nonbonded_method == MPID_PME;
        if (usePme) {
            if (!(s.ewald_alpha > 0) || s.grid[0] <= 0 || s.grid[1] <= 0 || s.grid[2] <= 0)
                throw Error(MPID_ERR_INVALID, "PME needs explicit ewald_alpha > 0 and grid dimensions > 0");
            if (s.pme_order != 5 && s.pme_order != 6)
                throw Error(MPID_ERR_INVALID, "pme_order must be 5 or 6");
            // a stencil wraps around the grid at most once
            if (s.grid[0] < s.pme_order || s.grid[1] < s.pme_order || s.grid[2] < s.pme_order)
                throw Error(MPID_ERR_INVALID, "each PME grid dimension must be at least the B-spline order");
            if (!(s.cutoff > 0)) throw Error(MPID_ERR_INVALID, "cutoff must be positive");
        }
        if (s.polarization_type == MPID_EXTRAPOLATED && (s.n_extrap < 1 || s.n_extrap > 8))
            throw Error(MPID_ERR_INVALID, "extrapolation needs 1..8 coefficients");
        mixed = s.precision == MPID_PRECISION_MIXED;
        CUDA_CHECK(cudaSetDevice(device));
        CUDA_CHECK(cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, device));
        numSMs = std::max(numSMs, 1);
        npad = ((n + 31) / 32) * 32;
        ntiles = npad / 32;
        charge.alloc(n); dipole.alloc(3 * n); quad.alloc(6 * n); oct.alloc(10 * n); thole.alloc(n); pol.alloc(3 * n);
        axis.alloc(n); az.alloc(n); ax.alloc(n); ay.alloc(n);
        keys.alloc(n); keysAlt.alloc(n); order.alloc(n); orderAlt.alloc(n);
        cub::DeviceRadixSort::SortPairs(nullptr, cubBytes, keys.p, keysAlt.p, order.p, orderAlt.p, n);
        cubTemp.alloc(cubBytes);
        pos.alloc(3 * n); wpos.alloc(3 * n); center.alloc(3 * ntiles); half.alloc(3 * ntiles);
        centerF.alloc(ntiles); halfF.alloc(ntiles);
        // list capacities from the density (regrown on overflow)
        tileCount.alloc(ntiles); countL.alloc(npad); countS.alloc(npad); loL.alloc(npad); loS.alloc(npad);
        tmaxL.alloc(ntiles); tmaxS.alloc(ntiles);
        listMax.alloc(4);
        alloc_tile_lists(usePme ? std::min(ntiles, 96) : ntiles);
        alloc_atom_lists(usePme ? 64 : npad);
        forceFx.alloc(3 * (size_t) npad); torqueFx.alloc(3 * (size_t) npad);
        mom64.alloc(20 * (size_t) npad); prm64.alloc(2 * (size_t) n);
        scaledPairs.alloc(1); scaledScale.alloc(1); scaledPartial.alloc(1);
        energyPartial.alloc(nblk(npad, 32)); energyOut.alloc(4);
        forcesOut.alloc(3 * (size_t) n);
        partial.alloc(2 * (size_t) nblk(npad, 256)); red.alloc(4); sc.alloc(8);
        iter.alloc(1); done.alloc(1);
        counters.alloc(3);
        CUDA_CHECK(cudaMemset(counters.p, 0, 3 * sizeof(unsigned)));
        // The reciprocal-space chain (spread, FFTs, convolution, gather) is the longer of
        // the two branches of every field evaluation, so its kernels get the highest
        // stream priority and take SMs ahead of the wide real-space pair kernels.
        int prLeast = 0, prGreatest = 0;
        CUDA_CHECK(cudaDeviceGetStreamPriorityRange(&prLeast, &prGreatest));
        CUDA_CHECK(cudaStreamCreateWithPriority(&pmeOwn, cudaStreamNonBlocking, prGreatest));
        CUDA_CHECK(cudaStreamCreateWithFlags(&hostStream, cudaStreamNonBlocking));
        if (s.precision == MPID_PRECISION_MIXED && s.polarization_type == MPID_MUTUAL) {
            CUDA_CHECK(cudaStreamCreateWithFlags(&refOwn, cudaStreamNonBlocking));
            CUDA_CHECK(cudaStreamCreateWithPriority(&refPmeOwn, cudaStreamNonBlocking, prGreatest));
            for (cudaEvent_t* e : {&evRefFork, &evRefJoin, &evRefStart, &evRefDone})
                CUDA_CHECK(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
            CUDA_CHECK(cudaMallocHost(&refHost, sizeof(double)));
        }
        CUDA_CHECK(cudaEventCreateWithFlags(&evFork, cudaEventDisableTiming));
        CUDA_CHECK(cudaEventCreateWithFlags(&evJoin, cudaEventDisableTiming));
        serialStages = (s.flags & MPID_FLAG_SERIAL_STAGES) != 0;
        bind_streams();
        CUDA_CHECK(cudaMallocHost(&hostDone, 260 * sizeof(int)));
        CUDA_CHECK(cudaMallocHost(&hostSc, 8 * sizeof(double)));
        CUDA_CHECK(cudaMallocHost(&hostMax, 4 * sizeof(int)));
        CUDA_CHECK(cudaEventCreateWithFlags(&evLists, cudaEventDisableTiming));
        CUDA_CHECK(cudaEventCreate(&evStart));
        CUDA_CHECK(cudaEventCreate(&evStop));
        timer.init();
        iterEvents.resize(256);
        for (auto& e : iterEvents) CUDA_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        const int nPT = s.polarization_type == MPID_EXTRAPOLATED ? s.n_extrap : 0;
        if (mixed) {
            ef.reset(new Engine<float>());
            ef->init(n, npad, usePme, s.pme_order, s.grid, numSMs);
            pack0.alloc(npad); pack1.alloc(npad);
            cgR = build_cg_radial(usePme ? s.ewald_alpha : 0.0, Prec<float>::kQuadX, list_cutoff());
            r32.alloc(3 * (size_t) npad); p32.alloc(3 * (size_t) npad); q32.alloc(3 * (size_t) npad);
            x32.alloc(3 * (size_t) npad); b32.alloc(3 * (size_t) npad); res32.alloc(3 * (size_t) npad);
            s32.alloc(3 * (size_t) npad);
            if (nPT) { ptMuF.alloc((size_t) nPT * 3 * npad); ptEF.alloc((size_t) nPT * 3 * npad); ptGF.alloc((size_t) nPT * 6 * npad); }
            if (s.polarization_type == MPID_MUTUAL) {
                ed.reset(new Engine<double>());  // FP64 residual of the refinement loop
                ed->init(n, npad, usePme, s.pme_order, s.grid, numSMs);
                offDF.alloc(3 * (size_t) npad); muDF.alloc(3 * (size_t) npad);
                tholeDF.alloc(npad); dampDF.alloc(npad);
                if (usePme) {
                    const double rq = Prec<float>::kQuadX / s.ewald_alpha;
                    const double rL = s.cutoff * (1.0 + 1e-6) + 1e-5;
                    build_ewald_tables(s.ewald_alpha, rq, rL, 32, 7, tabGh, tabHh);
                    upload(tabG, tabGh.coef); upload(tabGc, tabGh.centre);
                    upload(tabH, tabHh.coef); upload(tabHc, tabHh.centre);
                }
            }
        } else {
            ed.reset(new Engine<double>());
            ed->init(n, npad, usePme, s.pme_order, s.grid, numSMs);
            if (nPT) { ptMuD.alloc((size_t) nPT * 3 * npad); ptED.alloc((size_t) nPT * 3 * npad); ptGD.alloc((size_t) nPT * 6 * npad); }
        }
        if (s.polarization_type == MPID_MUTUAL) {
            r64.alloc(3 * (size_t) npad); p64.alloc(3 * (size_t) npad); q64.alloc(3 * (size_t) npad);
            y64.alloc(3 * (size_t) npad); b64.alloc(3 * (size_t) npad); res64.alloc(3 * (size_t) npad);
            s64.alloc(3 * (size_t) npad);
            Efix64.alloc(3 * (size_t) npad);
        }
        if (usePme) {
            std::vector<double> mx = bspline_moduli(s.pme_order, s.grid[0]);
            std::vector<double> my = bspline_moduli(s.pme_order, s.grid[1]);
            std::vector<double> mz = bspline_moduli(s.pme_order, s.grid[2]);
            modx.alloc(mx.size()); mody.alloc(my.size()); modz.alloc(mz.size());
            CUDA_CHECK(cudaMemcpy(modx.p, mx.data(), mx.size() * 8, cudaMemcpyHostToDevice));
            CUDA_CHECK(cudaMemcpy(mody.p, my.data(), my.size() * 8, cudaMemcpyHostToDevice));
            CUDA_CHECK(cudaMemcpy(modz.p, mz.data(), mz.size() * 8, cudaMemcpyHostToDevice));
            influence.alloc((size_t) s.grid[0] * s.grid[1] * (s.grid[2] / 2 + 1));
        }
        // empty covalent lists until set
        std::vector<int> off0(n + 1, 0);
        covOff.alloc(n + 1);
        CUDA_CHECK(cudaMemcpy(covOff.p, off0.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice));
        covJ.alloc(1);
        covS.alloc(1);
    }

    void set_multipoles(const double* q, const double* d, const double* Q, const double* O, const int* at, const int* z,
                        const int* x, const int* y, const double* th, const double* p) {
        // MPIDForceImpl::initialize validation (openmmapi/src/MPIDForceImpl.cpp:72-150)
        const double tol = 1.0e-5;
        for (int i = 0; i < n; ++i) {
            double tr = std::fabs(Q[6 * i] + Q[6 * i + 2] + Q[6 * i + 5]);
            if (tr > tol) {
                std::ostringstream m;
                m << "MPIDForce: quadrupole for particle=" << i << " has nonzero trace: " << tr
                  << "; MPID plugin assumes traceless quadrupole.";
                throw Error(MPID_ERR_INVALID, m.str());
            }
            const int tr3[3][3] = {{0, 2, 7}, {1, 3, 8}, {4, 6, 9}};
            const char* names[3] = {"(XXX,XYY,XZZ)", "(YXX,YYY,YZZ)", "(ZXX,ZYY,ZZZ)"};
            for (int k = 0; k < 3; ++k) {
                double t = std::fabs(O[10 * i + tr3[k][0]] + O[10 * i + tr3[k][1]] + O[10 * i + tr3[k][2]]);
                if (t > tol) {
                    std::ostringstream m;
                    m << "MPIDForce: " << names[k] << " octopole for particle=" << i << " has nonzero trace: " << t
                      << "; MPID plugin assumes traceless octopoles.";
                    throw Error(MPID_ERR_INVALID, m.str());
                }
            }
            if (at[i] < 0 || at[i] > NoAxisType) {
                std::ostringstream m;
                m << "MPIDForce: axis type=" << at[i] << " not currently handled";
                throw Error(MPID_ERR_INVALID, m.str());
            }
            if (at[i] != NoAxisType && (z[i] < 0 || z[i] >= n)) {
                std::ostringstream m;
                m << "MPIDForce: invalid z axis particle: " << z[i];
                throw Error(MPID_ERR_INVALID, m.str());
            }
            if (at[i] != NoAxisType && at[i] != ZOnly && (x[i] < 0 || x[i] >= n)) {
                std::ostringstream m;
                m << "MPIDForce: invalid x axis particle: " << x[i];
                throw Error(MPID_ERR_INVALID, m.str());
            }
            if ((at[i] == ZBisect || at[i] == ThreeFold) && (y[i] < 0 || y[i] >= n)) {
                std::ostringstream m;
                m << "MPIDForce: invalid y axis particle: " << y[i];
                throw Error(MPID_ERR_INVALID, m.str());
            }
            if (y[i] >= n) throw Error(MPID_ERR_INVALID, "MPIDForce: invalid y axis particle");
            for (int k = 0; k < 3; ++k)
                if (p[3 * i + k] < 0) throw Error(MPID_ERR_INVALID, "MPIDForce: negative polarizability");
        }
        h_axis.assign(at, at + n); h_az.assign(z, z + n); h_ax.assign(x, x + n); h_ay.assign(y, y + n);
        CUDA_CHECK(cudaMemcpy(charge.p, q, n * 8, cudaMemcpyHostToDevice));
        CUDA_CHECK(cudaMemcpy(dipole.p, d, 3 * n * 8, cudaMemcpyHostToDevice));
        CUDA_CHECK(cudaMemcpy(quad.p, Q, 6 * n * 8, cudaMemcpyHostToDevice));
        CUDA_CHECK(cudaMemcpy(oct.p, O, 10 * n * 8, cudaMemcpyHostToDevice));
        CUDA_CHECK(cudaMemcpy(thole.p, th, n * 8, cudaMemcpyHostToDevice));
        CUDA_CHECK(cudaMemcpy(pol.p, p, 3 * n * 8, cudaMemcpyHostToDevice));
        CUDA_CHECK(cudaMemcpy(axis.p, at, n * 4, cudaMemcpyHostToDevice));
        CUDA_CHECK(cudaMemcpy(az.p, z, n * 4, cudaMemcpyHostToDevice));
        CUDA_CHECK(cudaMemcpy(ax.p, x, n * 4, cudaMemcpyHostToDevice));
        CUDA_CHECK(cudaMemcpy(ay.p, y, n * 4, cudaMemcpyHostToDevice));
        haveParams = true;
    }

    // Pair scale from covalent maps as MPIDReferenceForce::setupScaleMaps
    // (MPIDReferenceForce.cpp:190-225): the lower-index atom's lists decide, types
    // 1-2, 1-3 -> 0, 1-4 -> scale14, 1-5 -> 1, later types overwrite earlier ones.
    void set_covalent(const int* offsets, const int* index) {
        const double sval[4] = {0.0, 0.0, set.scale14, 1.0};
        std::map<std::pair<int, int>, double> sc;
        for (int i = 0; i < n; ++i)
            for (int t = 0; t < 4; ++t)
                for (int k = offsets[8 * i + t]; k < offsets[8 * i + t + 1]; ++k) {
                    const int j = index[k];
                    if (j < 0 || j >= n) throw Error(MPID_ERR_INVALID, "MPIDForce: covalent index out of range");
                    if (j < i) continue;
                    sc[{i, j}] = sval[t];
                }
        std::vector<int2> sp;
        std::vector<double> ssc;
        for (auto& kv : sc)
            if (kv.second != 1.0 && kv.first.first != kv.first.second) {
                sp.push_back(make_int2(kv.first.first, kv.first.second));
                ssc.push_back(kv.second);
            }
        nScaled = (int) sp.size();
        scaledPairs.alloc(std::max(nScaled, 1));
        scaledScale.alloc(std::max(nScaled, 1));
        scaledPartial.alloc(std::max(nblk(nScaled, 128), 1));
        if (nScaled) {
            CUDA_CHECK(cudaMemcpy(scaledPairs.p, sp.data(), nScaled * sizeof(int2), cudaMemcpyHostToDevice));
            CUDA_CHECK(cudaMemcpy(scaledScale.p, ssc.data(), nScaled * sizeof(double), cudaMemcpyHostToDevice));
        }
        std::vector<std::vector<std::pair<int, double>>> lists(n);
        for (auto& kv : sc) {
            if (kv.second == 1.0 || kv.first.first == kv.first.second) continue;
            lists[kv.first.first].push_back({kv.first.second, kv.second});
            lists[kv.first.second].push_back({kv.first.first, kv.second});
        }
        std::vector<int> off(n + 1, 0), js;
        std::vector<double> ss;
        for (int i = 0; i < n; ++i) {
            for (auto& e : lists[i]) { js.push_back(e.first); ss.push_back(e.second); }
            off[i + 1] = (int) js.size();
        }
        covJ.alloc(std::max<size_t>(js.size(), 1));
        covS.alloc(std::max<size_t>(ss.size(), 1));
        CUDA_CHECK(cudaMemcpy(covOff.p, off.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice));
        if (!js.empty()) {
            CUDA_CHECK(cudaMemcpy(covJ.p, js.data(), js.size() * sizeof(int), cudaMemcpyHostToDevice));
            CUDA_CHECK(cudaMemcpy(covS.p, ss.data(), ss.size() * sizeof(double), cudaMemcpyHostToDevice));
        }
    }

    MolArrays mol() const {
        MolArrays m;
        m.charge = charge.p; m.dipole = dipole.p; m.quad = quad.p; m.oct = oct.p; m.thole = thole.p; m.pol = pol.p;
        m.axis = axis.p; m.az = az.p; m.ax = ax.p; m.ay = ay.p;
        return m;
    }

    void set_box(const double* b) {
        // OpenMM's reduced form: a = (ax, 0, 0), b = (bx, by, 0), c = (cx, cy, cz)
        if (b[1] != 0.0 || b[2] != 0.0 || b[5] != 0.0)
            throw Error(MPID_ERR_INVALID, "the periodic box must be in reduced form: a = (ax, 0, 0), b = (bx, by, 0)");
        const double L[3] = {b[0], b[4], b[8]};
        const bool tri = b[3] != 0.0 || b[6] != 0.0 || b[7] != 0.0;
        if (usePme) {
            for (int k = 0; k < 3; ++k)
                if (!(L[k] > 0)) throw Error(MPID_ERR_INVALID, "Box size of zero is invalid.");
            if (tri && (std::fabs(b[3]) > 0.5 * L[0] * (1 + 1e-12) || std::fabs(b[6]) > 0.5 * L[0] * (1 + 1e-12) ||
                        std::fabs(b[7]) > 0.5 * L[1] * (1 + 1e-12)))
                throw Error(MPID_ERR_INVALID, "the periodic box must be in reduced form: |bx|, |cx| <= ax/2, |cy| <= by/2");
            const double minAllowed = 1.999999 * set.cutoff;  // MPIDReferenceKernels.cpp:193-197
            if (L[0] < minAllowed || L[1] < minAllowed || L[2] < minAllowed)
                throw Error(MPID_ERR_INVALID, "The periodic box size has decreased to less than twice the nonbonded cutoff.");
        }
        for (int k = 0; k < 3; ++k) {
            box.L[k] = usePme ? L[k] : 1.0;
            box.invL[k] = usePme ? 1.0 / L[k] : 1.0;
            box.grid[k] = usePme ? set.grid[k] : 1;
        }
        for (int k = 0; k < 9; ++k) box.V[k] = usePme ? b[k] : ((k % 4) == 0 ? 1.0 : 0.0);
        box.tri = usePme && tri ? 1 : 0;
        // reciprocal vectors as MPIDReferenceForce.cpp:2627-2632 stores them
        const double* v = box.V;
        const double scale = 1.0 / (v[0] * v[4] * v[8]);
        const double R[3][3] = {{v[4] * v[8] * scale, 0.0, 0.0},
                                {-v[3] * v[8] * scale, v[0] * v[8] * scale, 0.0},
                                {(v[3] * v[7] - v[4] * v[6]) * scale, -v[0] * v[7] * scale, v[0] * v[4] * scale}};
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) box.R[i][j] = R[i][j];
        // fractional grid coordinates: frac_j = grid_j sum_i x_i R[i][j]
        for (int j = 0; j < 3; ++j)
            for (int i = 0; i < 3; ++i) box.A[j][i] = usePme ? set.grid[j] * R[i][j] : 0.0;
        if (usePme && std::memcmp(lastBox, b, sizeof(lastBox)) != 0) {
            const size_t Gh = (size_t) set.grid[0] * set.grid[1] * (set.grid[2] / 2 + 1);
            launch<k_influence>(std::min<long long>(nblk(Gh, 256), (long long) numSMs * 8), 256, 0, stream, box, set.ewald_alpha,
                   modx.p, mody.p, modz.p, L[0] * L[1] * L[2], influence.p);
            CUDA_CHECK(cudaGetLastError());
            std::memcpy(lastBox, b, sizeof(lastBox));
        }
    }

    void alloc_tile_lists(int c) {
        tcap = c;
        tileJ.alloc((size_t) ntiles * tcap);
        shF.alloc((size_t) ntiles * tcap);
        shD.alloc((size_t) 3 * ntiles * tcap);
        shDF.alloc((size_t) 3 * ntiles * tcap);
    }
    void alloc_atom_lists(int c) {
        cap = ((c + chunk - 1) / chunk) * chunk;
        const size_t entries = (size_t) npad * cap;
        if (entries > ((size_t) 1 << 34)) throw Error(MPID_ERR_INVALID, "neighbour list would exceed 64 GB");
        list.alloc(entries);
        listEntries = (long long) entries;
        // one entry per warp task; split tasks stay below twice the split target
        energyBlocks.alloc(std::max((size_t) ntiles * (cap / chunk + 2), (size_t) 4 * numSMs * 64));
    }

    static void upload(DBuf<float>& d, const std::vector<float>& h) {
        d.alloc(h.size());
        CUDA_CHECK(cudaMemcpy(d.p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    }

    DfRadial df_radial() const {
        DfRadial R;
        R.Gcoef = tabG.p; R.Gcentre = tabGc.p; R.Hcoef = tabH.p; R.Hcentre = tabHc.p;
        R.Gr0 = tabGh.r0; R.Ginvh = tabGh.invh; R.GK = tabGh.K;
        R.Hr0 = tabHh.r0; R.Hinvh = tabHh.invh; R.HK = tabHh.K;
        R.usePme = usePme ? 1 : 0;
        R.rc2 = usePme ? (float) (set.cutoff * set.cutoff) : 3.0e38f;
        for (int k = 0; k < 3; ++k) {
            R.L[k] = (float) box.L[k];
            R.iL[k] = (float) box.invL[k];
        }
        for (int k = 0; k < 9; ++k) {
            const dfloat v = df_from_double(box.V[k]);
            R.Vdf[k] = make_float2(v.hi, v.lo);
        }
        const dfloat th = df_from_double(set.default_thole);
        R.tholeDefault = make_float2(th.hi, th.lo);
        return R;
    }

    DfAtoms df_atoms() const {
        DfAtoms A;
        A.npad = npad;
        A.off = offDF.p;
        A.mu = muDF.p;
        A.thole = tholeDF.p;
        A.damp = dampDF.p;
        return A;
    }

    template <typename real>
    PairConsts<real> pair_consts_host() const {
        PairConsts<real> c;
        for (int k = 0; k < 3; ++k) {
            c.L[k] = (real) box.L[k];
            c.iL[k] = (real) box.invL[k];
        }
        for (int k = 0; k < 9; ++k) c.V[k] = (real) box.V[k];
        c.rc2 = usePme ? (real) (set.cutoff * set.cutoff) : (real) 3.0e38f;
        c.thole = (real) set.default_thole;
        c.ew = EwaldAlpha<real>(usePme ? set.ewald_alpha : 0.0);
        return c;
    }

    NbrList nbr_list() const {
        NbrList c;
        c.ntiles = ntiles;
        c.tcap = tcap;
        c.cap = cap;
        c.chunk = chunk;
        c.nchunksL = nchunksL;
        c.nchunksS = nchunksS;
        c.tileJ = tileJ.p;
        c.shF = shF.p;
        c.shD = shD.p;
        c.shDF = shDF.p;
        c.countL = countL.p;
        c.countS = countS.p;
        c.loL = loL.p;
        c.loS = loS.p;
        c.tmaxL = tmaxL.p;
        c.tmaxS = tmaxS.p;
        c.list = list.p;
        c.usePbc = usePme ? 1 : 0;
        c.split = 1;
        c.cf = pair_consts_host<float>();
        c.cd = pair_consts_host<double>();
        c.covOff = covOff.p;
        c.covJ = covJ.p;
        c.covS = covS.p;
        return c;
    }

    // warp tasks (tile, chunk) of the pair kernels
    int pair_tasks() const { return ntiles * (nchunksL + nchunksS); }
    int pair_blocks() const { return std::max(1, nblk(pair_tasks(), kWarpsPerBlock)); }
    // The field and energy pair kernels cut each work item into sub-ranges until the
    // launch holds two full waves of warps (the device's SMs x 64 resident warps): their per-pair
    // gathers are latency-bound, and one work item per warp leaves SMs idle (most of
    // them below a few thousand atoms).  The lists and results are the same.  Measured
    // on the 24,000-atom box: the CG pair kernel goes from 87 to 75 us per launch
    // (split 4); on a 660-atom box the FP32 CG field from 41 to 10 us.
    int splitCap = 0;  // upper bound of field_split() (0: none); mpid_set_work_split
    int field_split() const {
        const int cap = splitCap > 0 ? std::min(splitCap, chunk) : chunk;
        int split = 1;
        while (split < cap && (long long) pair_tasks() * split < 2LL * numSMs * 64) split *= 2;
        return split;
    }
    NbrList field_list() const {
        NbrList c = nbr_list();
        c.split = field_split();
        return c;
    }
    int field_blocks() const { return gradient_blocks(field_split()); }

    // Spatial sort (PME) or caller order (no cutoff), then tile centres and extents.
    void sort_and_tiles() {
        cudaStream_t st = stream;
        if (usePme) {
            // columns about (32 / density)^(1/3) wide
            const double vol = box.L[0] * box.L[1] * box.L[2];
            const double edge = std::cbrt(32.0 * vol / n);
            const int ncx = std::max(1, (int) std::lround(box.L[0] / edge));
            const int ncy = std::max(1, (int) std::lround(box.L[1] / edge));
            // key bits: the column index, then up to 16 bits of z (a quantum of L_z / 65536)
            int colBits = 1;
            while (colBits < 28 && (1LL << colBits) < (long long) ncx * ncy) ++colBits;
            const int zBits = std::min(16, 32 - colBits);
            launch<k_sort_keys>(nblk(n, 256), 256, 0, st, n, pos.p, box, ncx, ncy, zBits, keys.p, orderAlt.p, wpos.p);
            if (t_recorder) {
                // a recorded (fused multi-box) evaluation sorts each box in one block
                if (n > kBlockSortMax) throw Error(MPID_ERR_INVALID, "fused batch: a box has more than 4096 atoms");
                launch<k_sort_block>(1, 1024, 0, st, n, (const unsigned*) keys.p, (const int*) orderAlt.p, order.p);
            } else {
                ++t_library_calls;
                CUDA_CHECK(cub::DeviceRadixSort::SortPairs(cubTemp.p, cubBytes, keys.p, keysAlt.p, orderAlt.p, order.p, n,
                                                            0, colBits + zBits, st));
            }
        } else {
            // No periodic box: keep the caller's order (all pairs interact).
            launch<k_identity_order>(nblk(n, 256), 256, 0, st, n, (const double*) pos.p, order.p, wpos.p);
        }
        launch<k_tile_bounds>(nblk((long long) ntiles * 32, 128), 128, 0, st, n, ntiles, order.p, wpos.p, center.p,
               half.p, centerF.p, halfF.p);
    }

    double list_cutoff() const { return usePme ? set.cutoff * (1.0 + 1e-6) + 1e-5 : 1e30; }

    // Tile lists and per-atom lists from the sorted offsets of engine e; the list maxima
    // go to pinned host memory, read by finish_lists.
    template <typename real>
    void launch_lists(Engine<real>& e, bool record = true) {
        cudaStream_t st = stream;
        const double listCut = list_cutoff();
        const float cut2 = usePme ? (float) (listCut * listCut) : 3.0e38f;
        // erfc / quadrature segment boundary: alpha r = kQuadX
        const float quadR2 = usePme ? (float) std::pow(Prec<float>::kQuadX / set.ewald_alpha, 2) : 0.f;
        op_memset(listMax.p, 0, 4 * sizeof(int), st);
        launch<k_tile_list>(ntiles, 32 * kTileListWarps, 0, st, ntiles, center.p, centerF.p, halfF.p, box, listCut,
               usePme ? 1 : 0, tcap, tileCount.p, tileJ.p, shF.p, shD.p, shDF.p, listMax.p);
        launch<k_atom_list<real>>(ntiles, 32 * kListWarps, 0, st, ntiles, npad, (const real*) e.off.p,
               (const int*) e.orig.p, (const int*) e.rank.p, box, cut2, quadR2, usePme ? 1 : 0, tcap, tileCount.p, tileJ.p, shF.p, covOff.p,
               covJ.p, covS.p, cap, countL.p, countS.p, loL.p, loS.p, tmaxL.p, tmaxS.p, list.p, listMax.p + 1);
        op_copy(hostMax, listMax.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, st);
        if (record) CUDA_CHECK(cudaEventRecord(evLists, st));
    }

    // Waits for the list maxima (work queued after launch_lists keeps the GPU busy), grows
    // and rebuilds on overflow, and sizes the pair kernels' work items.
    template <typename real>
    void finish_lists(Engine<real>& e) {
        for (int attempt = 0; attempt < 3; ++attempt) {
            CUDA_CHECK(cudaEventSynchronize(evLists));
            const int mTiles = hostMax[0], mTotal = hostMax[1], mL = hostMax[2], mS = hostMax[3];
            lastTiles = mTiles;
            lastMaxList = mTotal;
            if (mTiles <= tcap && mTotal <= cap) {
                nchunksL = (mL + chunk - 1) / chunk;
                nchunksS = (mS + chunk - 1) / chunk;
                if (nchunksL + nchunksS == 0) nchunksL = 1;
                return;
            }
            if (growForbidden) {
                if (mTiles > tcap)
                    throw Error(MPID_ERR_INVALID, "mpid_evaluate_device_noalloc: the tile lists would have to grow (" +
                                                      std::to_string(mTiles) + " > " + std::to_string(tcap) +
                                                      " neighbour tiles); evaluate once with mpid_evaluate_device first");
                throw Error(MPID_ERR_INVALID, "mpid_evaluate_device_noalloc: an atom has " + std::to_string(mTotal) +
                                                  " neighbours, more than the " + std::to_string(cap) +
                                                  " that the static scratch holds for this system size");
            }
            if (mTiles > tcap) alloc_tile_lists(std::min(ntiles, mTiles + mTiles / 4 + 8));
            // with a truncated tile list the atom counts are low: size from the worst case
            if (mTotal > cap || mTiles > tcap) alloc_atom_lists(std::min(npad, std::max(mTotal + mTotal / 8 + chunk, cap)));
            launch_lists(e);
        }
        throw Error(MPID_ERR_CUDA, "neighbour list overflow");
    }

    template <typename real>
    void prepare_engine(Engine<real>& e, bool main) {
        cudaStream_t st = stream;
        launch<k_gather_atoms<real>>(nblk(npad, 128), 128, 0, st, n, npad, order.p, mol(), pos.p, wpos.p, center.p, e.arrays(),
                                                               main ? mom64.p : nullptr, main ? prm64.p : nullptr);
        if (usePme) {
            e.pme.set_stream(pmeStream);
            e.pme.bsplines(n, npad, order.p, wpos.p, box, st);
            // the refinement engine spreads induced dipoles only
            if (main) launch<k_frac_multipoles<real>>(nblk(npad, 128), 128, 0, st, npad, box, e.mom.p, e.mf.p);
        }
        CUDA_CHECK(cudaGetLastError());
    }

    // Forward FFT, convolution, inverse FFT of engine e's grid on the PME stream `ps`,
    // inside an open ST_PME interval.  Under MPID_FLAG_SERIAL_STAGES the two cuFFT
    // executions are timed as their own stage.
    template <typename real>
    void convolve(Engine<real>& e, const int* skip, cudaStream_t ps) {
        if (!serialStages) {
            e.pme.convolve(influence.p, skip, ps);
            return;
        }
        PmeStage<real>& p = e.pme;
        timer.end(ps);
        timer.begin(ST_FFT, ps);
        p.fft(true);
        timer.end(ps);
        timer.begin(ST_PME, ps);
        launch<k_convolve<real>>(std::min<long long>(nblk(p.Gh, 256), (long long) p.sms * 16), 256, 0, ps, p.Gh,
               (const double*) influence.p, p.cgrid.p, skip);
        timer.end(ps);
        timer.begin(ST_FFT, ps);
        p.fft(false);
        timer.end(ps);
        timer.begin(ST_PME, ps);
    }

    double self_coef() const {
        return usePme ? 4.0 / 3.0 * set.ewald_alpha * set.ewald_alpha * set.ewald_alpha / kSqrtPiRef : 0.0;
    }

    // Reciprocal part of the permanent field of engine e (phiP): spread of the 20
    // multipole components, FFTs and the 35-term gather.  It needs no neighbour lists, so
    // the set-up forks it onto the PME stream right after the atom frames and B-splines,
    // beside the sort's successors and the list build, and joins it (fixed_recip_join) at
    // the end of the set-up.
    template <typename real>
    void fixed_recip_fork(Engine<real>& e) {
        if (!usePme) return;
        fork_pme();
        cudaStream_t ps = pmeStream;
        timer.begin(ST_PME, ps);
        e.pme.template spread<20>(n, npad, box, e.mf.p, nullptr, ps);
        convolve(e, nullptr, ps);
        e.pme.template gather<35>(n, npad, box, e.phiP.p, nullptr, ps);
        timer.end(ps);
    }
    void fixed_recip_join() {
        if (usePme) join_pme();
    }

    // Permanent field -> Efix, muD, SE: the real-space pairs plus the reciprocal part that
    // the set-up computed (fixed_recip_fork).
    template <typename real>
    void fixed_field(Engine<real>& e) {
        cudaStream_t st = stream;
        op_memset(e.fieldFx.p, 0, 3 * (size_t) npad * 8, st);
        timer.begin(ST_FIXED_REAL, st);
        launch<k_fixed_field<real>>(field_blocks(), 32 * kWarpsPerBlock, 0, st, field_list(), e.arrays(), e.fieldFx.p);
        timer.end(st);
        launch<k_record_fixed<real>>(nblk(npad, 128), 128, 0, st, n, npad, box, self_coef(), e.fieldFx.p,
                                                               usePme ? e.phiP.p : nullptr, e.arrays(), e.Efix.p, e.muD.p,
                                                               e.SE.p);
        CUDA_CHECK(cudaGetLastError());
    }

    // Field (and optionally gradient) of dipoles mu: real + reciprocal + self -> E, G.
    template <typename real>
    void dipole_field(Engine<real>& e, const real* mu, real* E, real* G, const int* skip, int nterm = 4) {
        cudaStream_t st = stream;
        op_memset(e.fieldFx.p, 0, 3 * (size_t) npad * 8, st);
        if (usePme) {
            fork_pme();
            cudaStream_t ps = pmeStream;
            timer.begin(ST_PME, ps);
            launch<k_frac_dipoles<real>>(nblk(npad, 128), 128, 0, ps, npad, box, mu, e.mfd.p, skip);
            e.pme.template spread<4>(n, npad, box, e.mfd.p, skip, ps);
            convolve(e, skip, ps);
            if (nterm == 4)
                e.pme.template gather<4>(n, npad, box, e.phiT.p, skip, ps);
            else if (nterm == 10)
                e.pme.template gather<10>(n, npad, box, e.phiT.p, skip, ps);
            else
                e.pme.template gather<35>(n, npad, box, e.phiT.p, skip, ps);
            timer.end(ps);
        }
        // the FP64 field of the mixed path's residual refinement is timed on its own
        timer.begin(mixed && sizeof(real) == 8 ? ST_REFINE_REAL : ST_DIPOLE_REAL, st);
        if (mixed && sizeof(real) == 8) {
            // residual refinement: real-space part in double-float on the FP32 pipes
            launch<k_to_df>(nblk(3LL * npad, 256), 256, 0, st, 3 * npad, (const double*) mu, muDF.p);
            launch<k_dipole_field_df>(field_blocks(), 32 * kWarpsPerBlock, 0, st, field_list(), df_radial(), df_atoms(),
                   (const int*) e.orig.p, e.fieldFx.p);
        } else if (G) {
            op_memset(e.gradFx.p, 0, 6 * (size_t) npad * 8, st);
            launch<k_dipole_field<real, true, sizeof(real) == 8>>(field_blocks(), 32 * kWarpsPerBlock, 0, st, field_list(), e.arrays(), mu, e.fieldFx.p,
                                                                                     e.gradFx.p, skip);
        } else {
            launch<k_dipole_field<real, false, sizeof(real) == 8>>(field_blocks(), 32 * kWarpsPerBlock, 0, st, field_list(), e.arrays(), mu,
                                                                                      e.fieldFx.p, nullptr, skip);
        }
        timer.end(st);
        if (usePme) join_pme();
        launch<k_dipole_field_total<real>>(nblk(npad, 128), 128, 0, st, n, npad, box, self_coef(), e.fieldFx.p, e.gradFx.p,
                                                                     usePme ? e.phiT.p : nullptr, nterm, mu, E, G, skip);
        CUDA_CHECK(cudaGetLastError());
    }

    // One CG operator application: (p = r + beta p unless first), sp = S p, E = T sp
    // (real space, reciprocal, self), q = p - S E and p.q into sc[1].
    template <typename real>
    void cg_matvec(Engine<real>& e, const real* r, real* p, real* q, bool first) {
        cudaStream_t st = stream;
        const int nb = nblk(npad, 256);
        const bool packed = sizeof(real) == 4;  // FP32: packed-operand pair kernel
        launch<k_cg_direction_sroot<real>>(nblk(npad, 128), 128, 0, st, npad, box, e.sroot.p, sc.p, first ? 1 : 0, r,
               p, e.sp.p, usePme ? e.mfd.p : (real*) nullptr, (const typename Vec4<real>::type*) e.prm.p,
               packed ? (typename Vec4<real>::type*) pack1.p : nullptr, done.p);
        if (usePme) {
            fork_pme();
            cudaStream_t ps = pmeStream;
            timer.begin(ST_PME, ps);
            e.pme.template spread<4>(n, npad, box, e.mfd.p, done.p, ps);
            convolve(e, done.p, ps);
            e.pme.template gather<4>(n, npad, box, e.phiT.p, done.p, ps);
            timer.end(ps);
        }
        timer.begin(ST_DIPOLE_REAL, st);
        if (packed)
            launch<k_dipole_field_cg>(field_blocks(), 32 * kWarpsPerBlock, 0, st, field_list(), cgR, (const float4*) pack0.p,
                   (const float4*) pack1.p, npad, (const int*) e.orig.p, e.fieldFx.p, (const int*) done.p);
        else
            launch<k_dipole_field<real, false, sizeof(real) == 8>>(field_blocks(), 32 * kWarpsPerBlock, 0, st, field_list(),
                   e.arrays(), (const real*) e.sp.p, e.fieldFx.p, (unsigned long long*) nullptr, (const int*) done.p);
        timer.end(st);
        if (usePme) join_pme();
        launch<k_cg_matvec_finish<real>>(nb, 256, 0, st, n, npad, box, self_coef(), e.fieldFx.p,
               usePme ? (const real*) e.phiT.p : (const real*) nullptr, (const real*) e.sroot.p, (const real*) p,
               (const real*) e.sp.p, q, partial.p, counters.p, sc.p, (const int*) done.p);
    }

    // z = P r with the near-field preconditioner (first: also p = z, sc[0] = r.z).
    template <typename real>
    void precondition(Engine<real>& e, const real* r, real* p, bool first) {
        cudaStream_t st = stream;
        if (nchunksS > 0)
            launch<k_precond_field<real>>(std::max(1, nblk(ntiles * nchunksS, kWarpsPerBlock)), 32 * kWarpsPerBlock, 0, st,
                   nbr_list(), e.arrays(), r, e.precFx.p, (const int*) done.p);
        launch<k_precond_finish<real>>(nblk(npad, 256), 256, 0, st, n, npad, (const real*) e.sroot.p, e.precFx.p, r, e.zc.p,
               p, first ? 1 : 0, partial.p, counters.p + 2, sc.p, (const int*) done.p);
    }

    // Graph replay is used under PME (the configuration it is tested on), on a created
    // stream that is not itself being captured by the caller (the legacy default stream
    // cannot be captured; a capture cannot nest): otherwise the launches run directly.
    // Decided once per evaluation.
    bool graphsActive = false;
    // Evaluations whose shape keeps changing (a box rescaled every step, lists that change
    // length) would capture new graphs every time, which costs more than launching
    // directly: after captures in each of the last 5 evaluations, the next 32 launch
    // directly.  (Warm-up evaluations capture too, also when other contexts allocate.)
    unsigned captureHistory = 0;
    int graphPause = 0;
    bool graph_mode() const { return graphsActive; }
    void note_captures() {
        if (!graphsActive) return;
        captureHistory = (captureHistory << 1) | (stats.graph_captures > 0 ? 1u : 0u);
        if ((captureHistory & 0x1fu) == 0x1fu) {
            graphPause = 32;
            captureHistory = 0;
        }
    }
    void choose_graph_mode() {
        note_captures();  // the previous evaluation and its gradient passes
        graphsActive = false;
        stats.graph_captures = 0;
        stats.graph_replays = 0;
        if (graphPause > 0) {
            --graphPause;
            return;
        }
        // the no-allocation call creates no graphs (instantiating one allocates)
        if (!(set.flags & MPID_FLAG_GRAPH_SOLVER) || !usePme || growForbidden || stream == nullptr ||
            stream == cudaStreamLegacy || stream == cudaStreamPerThread)
            return;
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CUDA_CHECK(cudaStreamIsCapturing(stream, &cs));
        graphsActive = cs == cudaStreamCaptureStatusNone;
    }

    // One CG iteration: q = B p = p - S T S p, p.q, then the update and the scalars
    // (PCG: p from z = P r).  Launches only.
    // The direction vector s of the single-reduction CG (one per precision).
    template <typename real>
    real* cg_s_vector() { return sizeof(real) == 4 ? (real*) (void*) s32.p : (real*) (void*) s64.p; }

    // One single-reduction CG iteration (k_cgcg_* kernels): w = B r (real space beside the
    // reciprocal chain on the side stream, then the self term), delta and alpha, then the
    // update of p, s, x and r with gamma', beta' and the convergence test.  q holds w.
    template <typename real, typename xreal>
    void cgcg_iteration(Engine<real>& e, xreal* x, real* r, real* p, real* q, double target, int maxIter) {
        cudaStream_t st = stream;
        const int nb = nblk(npad, 256);
        const bool packed = sizeof(real) == 4;  // FP32: packed-operand pair kernel
        if (usePme) {
            fork_pme();
            cudaStream_t ps = pmeStream;
            timer.begin(ST_PME, ps);
            e.pme.template spread<4>(n, npad, box, e.mfd.p, done.p, ps);
            convolve(e, done.p, ps);
            e.pme.template gather<4>(n, npad, box, e.phiT.p, done.p, ps);
            timer.end(ps);
        }
        timer.begin(ST_DIPOLE_REAL, st);
        if (packed)
            launch<k_dipole_field_cg>(field_blocks(), 32 * kWarpsPerBlock, 0, st, field_list(), cgR, (const float4*) pack0.p,
                   (const float4*) pack1.p, npad, (const int*) e.orig.p, e.fieldFx.p, (const int*) done.p);
        else
            launch<k_dipole_field<real, false, sizeof(real) == 8>>(field_blocks(), 32 * kWarpsPerBlock, 0, st, field_list(),
                   e.arrays(), (const real*) e.sp.p, e.fieldFx.p, (unsigned long long*) nullptr, (const int*) done.p);
        timer.end(st);
        if (usePme) join_pme();
        launch<k_cgcg_finish<real>>(nb, 256, 0, st, n, npad, box, self_coef(), e.fieldFx.p,
               usePme ? (const real*) e.phiT.p : (const real*) nullptr, (const real*) e.sroot.p, (const real*) r,
               (const real*) e.sp.p, q, partial.p, counters.p, sc.p, (const int*) iter.p, (const int*) done.p);
        launch<k_cgcg_update<real, xreal>>(nb, 256, 0, st, n, npad, box, (const real*) e.sroot.p, sc.p, (const real*) q, p,
               cg_s_vector<real>(), x, r, e.sp.p, usePme ? e.mfd.p : (real*) nullptr,
               (const typename Vec4<real>::type*) e.prm.p, packed ? (typename Vec4<real>::type*) pack1.p : nullptr,
               partial.p, counters.p, target, iter.p, maxIter, done.p);
        CUDA_CHECK(cudaGetLastError());
    }

    template <typename real, typename xreal>
    void cg_iteration(Engine<real>& e, xreal* x, real* r, real* p, real* q, double target, int maxIter, bool first) {
        const bool pcg = (set.flags & MPID_FLAG_NEAR_FIELD_PCG) != 0;
        if (!pcg) {
            cgcg_iteration(e, x, r, p, q, target, maxIter);
            return;
        }
        cg_matvec(e, pcg ? (const real*) e.zc.p : (const real*) r, p, q, first);
        launch<k_cg_update_scalars<real, xreal>>(nblk(npad, 256), 256, 0, stream, n, npad, e.sroot.p, sc.p, p, q, x, r,
               partial.p, counters.p + 1, target, iter.p, maxIter, done.p, pcg ? 1 : 0);
        if (pcg) precondition(e, r, p, false);
        CUDA_CHECK(cudaGetLastError());
    }

    // Preconditioned CG on B y = b, B = I - S T S, in precision `real`; x accumulates in xreal.
    // Convergence: 48.033324 sqrt(|S r|^2/n) < target.  cg_begin queues the start (and,
    // with solver graphs, iteration 0) without waiting; cg_finish runs the iterations to
    // convergence and returns the number used.
    template <typename real, typename xreal>
    void cg_begin(Engine<real>& e, const real* b, xreal* x, real* r, real* p, real* q, double target, int maxIter) {
        cudaStream_t st = stream;
        const int nb = nblk(npad, 256);
        if (!(set.flags & MPID_FLAG_NEAR_FIELD_PCG)) {
            // single-reduction CG: r = b, x = p = s = 0, gamma, the test and the operator input
            const bool packed = sizeof(real) == 4;
            launch<k_cgcg_start<real, xreal>>(nb, 256, 0, st, n, npad, box, (const real*) e.sroot.p, b, x, r, p,
                   cg_s_vector<real>(), e.sp.p, usePme ? e.mfd.p : (real*) nullptr, (const typename Vec4<real>::type*) e.prm.p,
                   packed ? (typename Vec4<real>::type*) pack1.p : nullptr, partial.p, counters.p, sc.p, target, iter.p,
                   done.p);
            op_memset(e.fieldFx.p, 0, 3 * (size_t) npad * 8, st);  // cleared again by each finish
            CUDA_CHECK(cudaGetLastError());
            if (graph_mode() && maxIter > 1) cg_iteration(e, x, r, p, q, target, maxIter, true);
            return;
        }
        launch<k_cg_start<real, xreal>>(nb, 256, 0, st, npad, e.sroot.p, b, x, r, p, partial.p, nb);
        launch<k_reduce_partials>(1, 1024, 0, st, nb, 2, partial.p, red.p, nullptr);
        launch<k_cg_init_scalars>(1, 1, 0, st, sc.p, red.p, n, target, iter.p, done.p);
        op_memset(e.fieldFx.p, 0, 3 * (size_t) npad * 8, st);  // cleared again by each matvec
        if (set.flags & MPID_FLAG_NEAR_FIELD_PCG) {
            op_memset(e.precFx.p, 0, 3 * (size_t) npad * 8, st);  // cleared by each application
            precondition(e, r, p, true);
        }
        CUDA_CHECK(cudaGetLastError());
        if (graph_mode() && maxIter > 1) cg_iteration(e, x, r, p, q, target, maxIter, true);
    }

    template <typename real, typename xreal>
    int cg_finish(Engine<real>& e, const real* b, xreal* x, real* r, real* p, real* q, double target, int maxIter,
                  double* finalMetric) {
        cudaStream_t st = stream;
        if (graph_mode() && maxIter > 1) {
            // Chunks replayed from graphs: first the length the last solve needed, then two
            // at a time.  Every iteration kernel returns at once when `done` is set, so a
            // chunk that overshoots costs only its launches.
            const bool pcg = (set.flags & MPID_FLAG_NEAR_FIELD_PCG) != 0;
            int it = 1, len = predictedIters > 1 ? predictedIters - 1 : 4;
            std::vector<long long> key = graph_key(kSegChunk);
            const void* ptrs[] = {&e, b, x, r, p, q};
            const long long more[] = {maxIter, pcg ? 1 : 0};
            key_put(key, ptrs, sizeof ptrs);
            key_put(key, more, sizeof more);
            key_put(key, &target, sizeof target);
            while (it < maxIter) {
                len = std::min(len, maxIter - it);
                std::vector<long long> k = key;
                k.push_back(len);
                replay(k, [&] {
                    for (int i = 0; i < len; ++i) cg_iteration(e, x, r, p, q, target, maxIter, false);
                }, 6 * len + 2);
                it += len;
                CUDA_CHECK(cudaMemcpyAsync(hostDone, done.p, sizeof(int), cudaMemcpyDeviceToHost, st));
                CUDA_CHECK(cudaEventRecord(iterEvents[0], st));
                CUDA_CHECK(cudaEventSynchronize(iterEvents[0]));
                if (hostDone[0]) break;
                len = 2;
            }
        } else {
            for (int it = 0; it < maxIter; ++it) {
                cg_iteration(e, x, r, p, q, target, maxIter, it == 0);
                const int slot = it % (int) iterEvents.size();
                CUDA_CHECK(cudaMemcpyAsync(hostDone + (slot % 256), done.p, sizeof(int), cudaMemcpyDeviceToHost, st));
                CUDA_CHECK(cudaEventRecord(iterEvents[slot], st));
                // Check the previous iteration's flag while this one runs (one-iteration lag).
                if (it >= 1) {
                    const int prev = (it - 1) % (int) iterEvents.size();
                    CUDA_CHECK(cudaEventSynchronize(iterEvents[prev]));
                    if (hostDone[prev % 256]) break;
                }
            }
        }
        op_copy(hostDone + 256, iter.p, sizeof(int), cudaMemcpyDeviceToHost, st);
        op_copy(hostSc, sc.p, 8 * sizeof(double), cudaMemcpyDeviceToHost, st);
        CUDA_CHECK(cudaStreamSynchronize(st));
        const int used = hostDone[256];
        if (finalMetric) *finalMetric = hostSc[6];
        predictedIters = used;
        return used;
    }

    template <typename real, typename xreal>
    int cg_solve(Engine<real>& e, const real* b, xreal* x, real* r, real* p, real* q, double target, int maxIter,
                 double* finalMetric) {
        cg_begin(e, b, x, r, p, q, target, maxIter);
        return cg_finish(e, b, x, r, p, q, target, maxIter, finalMetric);
    }

    // ----- CUDA graphs (MPID_FLAG_GRAPH_SOLVER) -----
    // Segments of an evaluation between host synchronisations are captured once and
    // replayed.  A graph is found by a key of 64-bit words holding every value its
    // launches bake in: the segment, the device-buffer generation (any reallocation
    // anywhere changes it), the list buffers (the no-alloc call points them at its
    // scratch), the list shape and launch sizes, the box and the constants.
    enum { kSegChunk = 1, kSegSetup, kSegSolveStart, kSegFinish, kSegGradients, kSegFull };

    static void key_put(std::vector<long long>& k, const void* v, size_t bytes) {
        const size_t o = k.size();
        k.resize(o + (bytes + 7) / 8, 0);
        std::memcpy(k.data() + o, v, bytes);
    }

    std::vector<long long> graph_key(int segment) const {
        std::vector<long long> k;
        const long long ints[] = {segment, (long long) g_device_allocs.load(), n, npad, ntiles, tcap, cap, chunk,
                                  nchunksL, nchunksS, field_split(), field_blocks(), nScaled, mixed ? 1 : 0,
                                  usePme ? 1 : 0, (long long) energyBlocks.n, (long long) list.n};
        key_put(k, ints, sizeof ints);
        const void* ptrs[] = {list.p, energyBlocks.p};
        key_put(k, ptrs, sizeof ptrs);
        const double dbl[] = {self_coef(), set.ewald_alpha, set.cutoff, set.default_thole, set.mutual_eps};
        key_put(k, dbl, sizeof dbl);
        static_assert(sizeof(BoxDev) == 33 * sizeof(double) + 4 * sizeof(int), "BoxDev has padding");
        key_put(k, &box, sizeof box);
        return k;
    }

    // Runs `body` (launches only: no host synchronisation, allocation or host-side state
    // that a replay would skip) directly, or with graphs from the graph of `key`,
    // capturing it on first use.
    template <typename Body>
    void replay(const std::vector<long long>& key, Body&& body, int timedPairs = 24) {
        if (!graph_mode()) {
            body();
            return;
        }
        const SolverGraph& g = solver_graph(key, body, timedPairs);
        CUDA_CHECK(cudaGraphLaunch(g.exec, stream));
        ++stats.graph_replays;
        t_launches += g.nodes;
        t_library_calls += g.library;
        timer.replayed.insert(timer.replayed.end(), g.pairs.begin(), g.pairs.end());
    }

    // The graph of `key`, captured by running `body` on the main stream under stream
    // capture (side streams join the capture through the fork/join events and must be
    // joined back by the end of `body`).  At most eight graphs are kept; the least
    // recently used goes.
    template <typename Body>
    const SolverGraph& solver_graph(const std::vector<long long>& key, Body&& body, int timedPairs) {
        for (auto& g : graphs)
            if (g.key == key) {
                g.used = ++graphClock;
                return g;
            }
        cudaStream_t st = stream;
        ++stats.graph_captures;
        SolverGraph g;
        g.key = key;
        g.events.resize(2 * (size_t) timedPairs);
        for (auto& ev : g.events) CUDA_CHECK(cudaEventCreate(&ev));
        const long long l0 = t_launches, c0 = t_library_calls;
        cudaGraph_t graph = nullptr;
        auto stop_timing = [&] {
            timer.capPool = nullptr;
            timer.capPairs = nullptr;
            timer.capOpen.stage = -1;
        };
        cudaError_t ce = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
        if (ce != cudaSuccess) {
            g.destroy();
            CUDA_CHECK(ce);
        }
        timer.capPool = &g.events;
        timer.capPairs = &g.pairs;
        timer.capNext = 0;
        try {
            body();
        } catch (...) {
            stop_timing();
            cudaStreamEndCapture(st, &graph);
            if (graph) cudaGraphDestroy(graph);
            (void) cudaGetLastError();
            g.destroy();
            t_launches = l0;
            t_library_calls = c0;
            throw;
        }
        stop_timing();
        ce = cudaStreamEndCapture(st, &graph);
        g.nodes = t_launches - l0;
        g.library = t_library_calls - c0;
        t_launches = l0;  // counted when replayed
        t_library_calls = c0;
        if (ce == cudaSuccess) ce = cudaGraphInstantiate(&g.exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (ce != cudaSuccess) {
            g.destroy();
            CUDA_CHECK(ce);
        }
        g.used = ++graphClock;
        if (graphs.size() < 8) {
            graphs.push_back(std::move(g));
            return graphs.back();
        }
        auto lru = std::min_element(graphs.begin(), graphs.end(),
                                    [](const SolverGraph& x, const SolverGraph& y) { return x.used < y.used; });
        lru->destroy();
        *lru = std::move(g);
        return *lru;
    }

    template <typename real>
    void alpha_times(Engine<real>& e, const real* E, real* out) {
        launch<k_alpha_times<real>>(nblk(npad, 128), 128, 0, stream, npad, e.alab.p, E, out);
    }

    // Induced dipoles into e.mu (sorted) for the configured polarisation type.
    template <typename real>
    void solve_dipoles(Engine<real>& e, real* ptMu, real* ptE, real* ptG) {
        cudaStream_t st = stream;
        const size_t n3 = 3 * (size_t) npad;
        stats.solver_iterations = 0;
        stats.refinement_steps = 0;
        stats.solver_residual = 0.0;
        if (set.polarization_type == MPID_DIRECT) {
            op_copy(e.mu.p, e.muD.p, n3 * sizeof(real), cudaMemcpyDeviceToDevice, st);
            return;
        }
        if (set.polarization_type == MPID_EXTRAPOLATED) {
            // mu_0 = alpha E_fixed; mu_(m+1) = alpha E[mu_m]; mu = sum_m cbar_m mu_m
            // (MPIDReferenceForce.cpp:1125-1180).
            const int nPT = set.n_extrap;
            double cbar[8];
            for (int i = 0; i < nPT; ++i) {
                cbar[i] = 0.0;
                for (int j = i; j < nPT; ++j) cbar[i] += set.extrap_coeffs[j];
            }
            op_copy(ptMu, e.muD.p, n3 * sizeof(real), cudaMemcpyDeviceToDevice, st);
            for (int m = 0; m + 1 < nPT; ++m) {
                dipole_field(e, ptMu + m * n3, ptE + m * n3, ptG + m * 2 * n3, nullptr, 10);
                alpha_times(e, ptE + m * n3, ptMu + (m + 1) * n3);
            }
            op_memset(e.mu.p, 0, n3 * sizeof(real), st);
            for (int m = 0; m < nPT; ++m)
                launch<k_axpy<real>>(nblk((long long) n3, 256), 256, 0, st, (int) n3, real(cbar[m]), ptMu + m * n3, e.mu.p);
            stats.solver_iterations = nPT - 1;
            CUDA_CHECK(cudaGetLastError());
            return;
        }
        throw Error(MPID_ERR_STATE, "mutual solve dispatched to the generic path");
    }

    void solve_mutual_double(Engine<double>& e) {
        double metric = 0.0;
        int it = cg_solve<double, double>(e, e.SE.p, y64.p, r64.p, p64.p, q64.p, set.mutual_eps, set.max_iter, &metric);
        stats.solver_iterations = it;
        stats.solver_residual = metric;
        launch<k_mu_from_y<double, double>>(nblk(npad, 128), 128, 0, stream, npad, e.sroot.p, y64.p, e.mu.p);
        if (!(metric < set.mutual_eps)) not_converged(it, metric);
    }

    // Mixed precision: FP32 CG inner solves, FP64 residual and accumulation of y.
    // solve_mutual_mixed runs the first inner solve, sets the dipoles from it and launches
    // the FP64 residual check on the refinement streams without waiting; the caller runs
    // the force/energy phase meanwhile and then calls finish_mutual_mixed, which waits for
    // the check and, if the residual misses the target, continues the outer iterations
    // (returning false: the force/energy phase must run again).
    void solve_mutual_mixed(Engine<float>& e, Engine<double>& d) {
        mutual_mixed_start(e);
        refOuter = 0;
        refTotal = 0;
        inner_solve_and_check(e, d);
    }

    // FP64 permanent field for the residual, y = 0, b = S E (launches only).
    void mutual_mixed_start(Engine<float>& e) {
        cudaStream_t st = stream;
        const size_t n3 = 3 * (size_t) npad;
        op_memset(Efix64.p, 0, n3 * 8, st);
        launch<k_axpy_to_double<float>>(nblk((long long) n3, 256), 256, 0, st, (int) n3, e.Efix.p, Efix64.p);
        op_memset(y64.p, 0, n3 * 8, st);
        op_copy(b32.p, e.SE.p, n3 * 4, cudaMemcpyDeviceToDevice, st);
    }

    // inner FP32 solves stop at half the target: the FP64 residual then meets the target
    // with a 2x margin for the FP32 operator's rounding (water24k: 9 iterations, final
    // FP64 residual 4.3e-8 D for a 1e-7 D target)
    double inner_target() const { return 0.5 * set.mutual_eps; }

    // One outer step: inner FP32 solve from b32, y += x, dipoles from y on the main
    // stream, and the FP64 residual S (E + T S y) - y launched on the refinement streams.
    void inner_solve_and_check(Engine<float>& e, Engine<double>& d) {
        const int maxIter = std::max(1, set.max_iter - refTotal);
        refTotal += cg_solve<float, float>(e, b32.p, x32.p, r32.p, p32.p, q32.p, inner_target(), maxIter, nullptr);
        launch_check(e, d);
        ++refOuter;
    }

    // y += x, the dipoles from y, and the FP64 residual check on the refinement streams,
    // which ends with evRefDone recorded there (launches only).
    void launch_check(Engine<float>& e, Engine<double>& d) {
        cudaStream_t st = stream;
        const int nb = nblk(npad, 256);
        const size_t n3 = 3 * (size_t) npad;
        launch<k_axpy_to_double<float>>(nblk((long long) n3, 256), 256, 0, st, (int) n3, x32.p, y64.p);
        launch<k_mu_from_y<double, float>>(nblk(npad, 128), 128, 0, st, npad, d.sroot.p, y64.p, e.mu.p);
        op_record(evRefStart, st);
        // the check, on the refinement streams (members swapped for the launches)
        RefStreams scope(*this);
        cudaStream_t rs = stream;
        op_wait(rs, evRefStart);
        if (usePme) d.pme.set_stream(pmeStream);
        launch<k_mu_from_y<double, double>>(nblk(npad, 128), 128, 0, rs, npad, d.sroot.p, y64.p, d.mu.p);
        dipole_field(d, d.mu.p, d.Etmp.p, (double*) nullptr, nullptr, 4);
        launch<k_refine_residual>(nb, 256, 0, rs, npad, d.sroot.p, Efix64.p, d.Etmp.p, y64.p, res64.p, res32.p, partial.p);
        launch<k_reduce_partials>(1, 1024, 0, rs, nb, 1, partial.p, red.p, nullptr);
        op_copy(refHost, red.p, 8, cudaMemcpyDeviceToHost, rs);
        op_record(evRefDone, rs);
    }

    // The refinement streams and their fork/join events take the place of the main ones
    // for the scope (also when a launch throws), so that the FP64 check's launches go
    // through the same helpers as the main path's.
    void swap_ref() {
        std::swap(stream, refStream);
        std::swap(pmeStream, refPmeStream);
        std::swap(evFork, evRefFork);
        std::swap(evJoin, evRefJoin);
    }
    struct RefStreams {
        Context& c;
        explicit RefStreams(Context& x) : c(x) { c.swap_ref(); }
        ~RefStreams() { c.swap_ref(); }
        RefStreams(const RefStreams&) = delete;
        RefStreams& operator=(const RefStreams&) = delete;
    };

    // The mixed Mutual evaluation from the permanent field on, as three captured segments
    // and two host waits: (permanent field, solver start, iteration 0) | iterations | (check
    // on the refinement streams beside the force/energy phase, joined at the end).  The
    // rare second outer step runs as in the direct flow.
    void mutual_mixed_graphs(Engine<float>& e, Engine<double>& d) {
        const int maxIter = std::max(1, set.max_iter);
        replay(graph_key(kSegSolveStart), [&] {
            fixed_field(e);
            mutual_mixed_start(e);
            cg_begin<float, float>(e, b32.p, x32.p, r32.p, p32.p, q32.p, inner_target(), maxIter);
        });
        refOuter = 0;
        refTotal = cg_finish<float, float>(e, b32.p, x32.p, r32.p, p32.p, q32.p, inner_target(), maxIter, nullptr);
        replay(graph_key(kSegFinish), [&] {
            launch_check(e, d);
            finish(e, ptMuF.p, ptEF.p, ptGF.p);
            CUDA_CHECK(cudaStreamWaitEvent(stream, evRefDone, 0));
        });
        ++refOuter;
        CUDA_CHECK(cudaEventRecord(evRefDone, stream));  // the check's result is in refHost once this passes
        if (!finish_mutual_mixed(e, d)) finish(e, ptMuF.p, ptEF.p, ptGF.p);
    }

    // Wait for the pending check; true if the dipoles the force/energy phase used stand.
    bool finish_mutual_mixed(Engine<float>& e, Engine<double>& d) {
        bool rerun = false;
        for (;;) {
            CUDA_CHECK(cudaEventSynchronize(evRefDone));
            const double metric = 48.033324 * std::sqrt(*refHost / n);
            stats.refinement_steps = refOuter;
            stats.solver_iterations = refTotal;
            stats.solver_residual = metric;
            if (metric < set.mutual_eps) return !rerun;
            if (refOuter >= 6 || refTotal >= set.max_iter || !(metric == metric)) not_converged(refTotal, metric);
            // continue from the residual: the main stream waits for the check's outputs
            CUDA_CHECK(cudaStreamWaitEvent(stream, evRefDone, 0));
            CUDA_CHECK(cudaMemcpyAsync(b32.p, res32.p, 3 * (size_t) npad * 4, cudaMemcpyDeviceToDevice, stream));
            inner_solve_and_check(e, d);
            rerun = true;
        }
    }

    [[noreturn]] void not_converged(int it, double eps) {
        std::ostringstream m;
        m << "Induced dipoles did not converge:  iterations=" << it << " eps=" << eps;
        throw Error(MPID_ERR_NOT_CONVERGED, m.str());
    }

    template <typename real>
    void finish(Engine<real>& e, real* ptMu, real* ptE, real* ptG) {
        cudaStream_t st = stream;
        op_memset(forceFx.p, 0, 3 * (size_t) npad * 8, st);
        op_memset(torqueFx.p, 0, 3 * (size_t) npad * 8, st);
        const NbrList tc = field_list();
        const int eb = pair_tasks() * tc.split;
        if ((size_t) eb > energyBlocks.n) throw Error(MPID_ERR_CUDA, "energy partials too small");
        op_memset(energyBlocks.p, 0, eb * sizeof(double), st);
        // The per-atom reciprocal/self terms and the FP64 energies of the covalently scaled
        // pairs run on the side stream after the reciprocal potential of the final induced
        // dipoles, beside the energy/force pair kernel on the main stream; both add into
        // the same fixed-point force and torque accumulators (integer atomics: the sums do
        // not depend on the order).
        fork_pme();
        cudaStream_t ps = pmeStream;
        if (usePme) {
            timer.begin(ST_PME, ps);
            launch<k_frac_dipoles<real>>(nblk(npad, 128), 128, 0, ps, npad, box, e.mu.p, e.mfd.p, nullptr);
            e.pme.template spread<4>(n, npad, box, e.mfd.p, nullptr, ps);
            convolve(e, nullptr, ps);
            e.pme.template gather<35>(n, npad, box, e.phiD.p, nullptr, ps);
            timer.end(ps);
        }
        timer.begin(ST_FINISH, ps);
        OptArgs opt{};
        if (set.polarization_type == MPID_EXTRAPOLATED) {
            opt.nPT = set.n_extrap;
            for (int i = 0; i < opt.nPT; ++i) {
                opt.cbar[i] = 0.0;
                for (int j = i; j < opt.nPT; ++j) opt.cbar[i] += set.extrap_coeffs[j];
            }
            opt.mu = ptMu;
            opt.E = ptE;
            opt.G = ptG;
        }
        // per-atom work is long: blocks small enough that a small system spans the SMs
        const int rb = npad >= 256 * 2 * numSMs ? 256 : (npad >= 128 * numSMs ? 128 : (npad >= 64 * numSMs ? 64 : 32));
        const int nb = nblk(npad, rb);
        launch<k_recip_self<real>>(nb, rb, 0, ps, n, npad, box, set.ewald_alpha, set.polarization_type,
               usePme ? e.phiP.p : nullptr, e.phiD.p, e.mu.p, e.arrays(), mom64.p, opt, forceFx.p, torqueFx.p,
               energyPartial.p);
        launch<k_reduce_partials>(1, 1024, 0, ps, nb, 1, energyPartial.p, energyOut.p, nullptr);
        if (nScaled) {
            const int sb = nblk(nScaled, 128);
            const int muIsFloat = sizeof(real) == 4 ? 1 : 0;
            if (set.polarization_type == MPID_MUTUAL)
                launch<k_scaled_pair_energy<true>>(sb, 128, 0, ps, nScaled, scaledPairs.p, scaledScale.p, e.rank.p, npad,
                       mom64.p, prm64.p, e.mu.p, muIsFloat, pos.p, box, usePme ? 1 : 0, set.cutoff,
                       usePme ? set.ewald_alpha : 0.0, set.default_thole, scaledPartial.p);
            else
                launch<k_scaled_pair_energy<false>>(sb, 128, 0, ps, nScaled, scaledPairs.p, scaledScale.p, e.rank.p, npad,
                       mom64.p, prm64.p, e.mu.p, muIsFloat, pos.p, box, usePme ? 1 : 0, set.cutoff,
                       usePme ? set.ewald_alpha : 0.0, set.default_thole, scaledPartial.p);
            launch<k_reduce_partials>(1, 1024, 0, ps, sb, 1, scaledPartial.p, energyOut.p + 2, nullptr);
        } else {
            op_memset(energyOut.p + 2, 0, sizeof(double), ps);
        }
        timer.end(ps);
        timer.begin(ST_PAIR, st);
        const bool exact = (set.flags & MPID_FLAG_EXACT_ANISO_TORQUE) != 0;
        const AtomArrays<real> aa = e.arrays();
        if (set.polarization_type == MPID_MUTUAL && !exact)
            launch<k_electrostatics<real, true, true, true>>(field_blocks(), 32 * kWarpsPerBlock, 0, st, tc, aa, e.mu.p, forceFx.p,
                                                                                             torqueFx.p, energyBlocks.p);
        else if (set.polarization_type == MPID_MUTUAL)
            launch<k_electrostatics<real, true, false, true>>(field_blocks(), 32 * kWarpsPerBlock, 0, st, tc, aa, e.mu.p, forceFx.p,
                                                                                              torqueFx.p, energyBlocks.p);
        else
            launch<k_electrostatics<real, false, true, true>>(field_blocks(), 32 * kWarpsPerBlock, 0, st, tc, aa, e.mu.p, forceFx.p,
                                                                                              torqueFx.p, energyBlocks.p);
        timer.end(st);
        join_pme();
        timer.begin(ST_FINISH, st);
        launch<k_reduce_partials>(1, 1024, 0, st, eb, 1, energyBlocks.p, energyOut.p + 1, nullptr);
        launch<k_torque_map>(nblk(n, 128), 128, 0, st, n, npad, pos.p, mol(), e.rank.p, torqueFx.p, forceFx.p);
        timer.end(st);
        CUDA_CHECK(cudaGetLastError());
    }

    template <typename real>
    int* rank_of(Engine<real>& e) { return e.rank.p; }

    // Full evaluation; d_pos / d_forces are device pointers.  Returns energy.
    double evaluate_device(const double* d_pos, const double* hbox, double* d_forces, double* d_energy) {
        if (!haveParams) throw Error(MPID_ERR_STATE, "mpid_set_multipoles must be called before evaluating");
        CUDA_CHECK(cudaSetDevice(device));
        bind_streams();
        cudaStream_t st = stream;
        choose_graph_mode();
        const long long launches0 = t_launches, library0 = t_library_calls;
        CUDA_CHECK(cudaEventRecord(evStart, st));
        if (d_pos != pos.p) CUDA_CHECK(cudaMemcpyAsync(pos.p, d_pos, 3 * (size_t) n * 8, cudaMemcpyDeviceToDevice, st));
        timer.reset();
        timer.begin(ST_SETUP, st);
        set_box(hbox);
        if (mixed) {
            Engine<float>& e = *ef;
            replay(graph_key(kSegSetup), [&] {
                sort_and_tiles();
                prepare_engine(e, true);
                fixed_recip_fork(e);  // beside the list build
                launch<k_pack_atoms>(nblk(npad, 128), 128, 0, st, npad, (const float*) e.off.p, (const float4*) e.prm.p,
                       pack0.p);
                if (ed) {
                    // the FP64 engine of the residual check is prepared on the check's stream,
                    // beside the list build (it is first read by the check)
                    op_record(evRefStart, st);
                    op_wait(refStream, evRefStart);
                    {
                        RefStreams scope(*this);
                        prepare_engine(*ed, false);
                        launch<k_df_atoms>(nblk(npad, 128), 128, 0, stream, npad, ed->off.p, ed->prm.p, offDF.p,
                               tholeDF.p, dampDF.p);
                    }
                    if (graph_mode()) {  // a captured side stream joins back before the capture ends
                        op_record(evRefStart, refStream);
                        op_wait(st, evRefStart);
                    }
                }
                launch_lists(e, false);
                fixed_recip_join();
            });
            CUDA_CHECK(cudaEventRecord(evLists, st));
            finish_lists(e);
            listsInScratch = growForbidden;
            stats.max_neighbours = lastMaxList;
            timer.end(st);
            if (set.polarization_type == MPID_MUTUAL && graph_mode()) {
                mutual_mixed_graphs(e, *ed);
            } else if (set.polarization_type == MPID_MUTUAL) {
                fixed_field(e);
                solve_mutual_mixed(e, *ed);
                finish(e, ptMuF.p, ptEF.p, ptGF.p);  // concurrent with the residual check
                if (!finish_mutual_mixed(e, *ed)) finish(e, ptMuF.p, ptEF.p, ptGF.p);
            } else {
                fixed_field(e);
                solve_dipoles(e, ptMuF.p, ptEF.p, ptGF.p);
                finish(e, ptMuF.p, ptEF.p, ptGF.p);
            }
            launch<k_forces_out>(nblk(n, 128), 128, 0, st, n, npad, e.rank.p, forceFx.p, d_forces);
        } else {
            Engine<double>& e = *ed;
            sort_and_tiles();
            prepare_engine(e, true);
            fixed_recip_fork(e);  // beside the list build
            launch_lists(e);
            fixed_recip_join();
            finish_lists(e);
            listsInScratch = growForbidden;
            stats.max_neighbours = lastMaxList;
            timer.end(st);
            fixed_field(e);
            if (set.polarization_type == MPID_MUTUAL)
                solve_mutual_double(e);
            else
                solve_dipoles(e, ptMuD.p, ptED.p, ptGD.p);
            finish(e, ptMuD.p, ptED.p, ptGD.p);
            launch<k_forces_out>(nblk(n, 128), 128, 0, st, n, npad, e.rank.p, forceFx.p, d_forces);
        }
        CUDA_CHECK(cudaGetLastError());
        double eparts[3] = {0, 0, 0};  // reciprocal + self, real space, scaled pairs
        CUDA_CHECK(cudaMemcpyAsync(eparts, energyOut.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaEventRecord(evStop, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
        const double energy = eparts[0] + eparts[1] + eparts[2];
        stats.energy_parts[0] = eparts[0];
        stats.energy_parts[1] = eparts[1];
        stats.energy_parts[2] = eparts[2];
        if (d_energy) CUDA_CHECK(cudaMemcpyAsync(d_energy, &energy, 8, cudaMemcpyHostToDevice, st));
        float ms = 0.f;
        CUDA_CHECK(cudaEventElapsedTime(&ms, evStart, evStop));
        stats.ms_total = ms;
        stats.kernel_launches = (int) (t_launches - launches0);
        stats.library_calls = (int) (t_library_calls - library0);
        timer.collect();
        for (int s = 0; s < ST_COUNT; ++s) {
            stats.ms_stage[s] = timer.ms[s];
            stats.stage_launches[s] = timer.launches[s];
        }
        evaluated = true;
        gradPrepared = false;
        CUDA_CHECK(cudaStreamSynchronize(st));
        return energy;
    }

    // ----- batched evaluation (mpid_evaluate_batch) -----
    // One complete evaluation (set-up, permanent field, induced dipoles, forces and
    // energy, optionally the gradient passes) captured as a graph with no host
    // synchronisation, so that the graphs of many contexts run as one launch.  The values
    // an ordinary evaluation decides on the host between its segments come from the
    // previous evaluation of the context: the list capacities, work-item counts and launch
    // sizes, and the number of CG iterations (the last solve's plus one).  The graph
    // copies to pinned host memory what decides whether its results stand -- the list
    // maxima, the solver's done flag, iteration count and metric, the FP64 residual of the
    // mixed path -- and batch_ok() checks them after the launch.
    struct FullGraph {
        std::vector<long long> key;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;  // for launches of this context's graph on its own
        long long nodes = 0, library = 0;
        int K = 0;
        unsigned long long generation = 0;  // changes with every capture
        void destroy() {
            if (exec) cudaGraphExecDestroy(exec);
            if (graph) cudaGraphDestroy(graph);
            exec = nullptr;
            graph = nullptr;
            key.clear();
        }
    } full;
    double* hostEparts = nullptr;  // pinned: the energy parts of a batched evaluation
    bool batchReady = false;       // an ordinary evaluation has sized the lists and the solver

    // The captured body (launches only).
    void batch_body(bool mg, bool pg, int K) {
        cudaStream_t st = stream;
        if (mixed) {
            Engine<float>& e = *ef;
            sort_and_tiles();
            prepare_engine(e, true);
            fixed_recip_fork(e);  // beside the list build
            launch<k_pack_atoms>(nblk(npad, 128), 128, 0, st, npad, (const float*) e.off.p, (const float4*) e.prm.p,
                   pack0.p);
            if (ed) {
                op_record(evRefStart, st);
                op_wait(refStream, evRefStart);
                {
                    RefStreams scope(*this);
                    prepare_engine(*ed, false);
                    launch<k_df_atoms>(nblk(npad, 128), 128, 0, stream, npad, ed->off.p, ed->prm.p, offDF.p, tholeDF.p,
                           dampDF.p);
                }
                op_record(evRefStart, refStream);
                op_wait(st, evRefStart);
            }
            launch_lists(e, false);  // the list maxima go to hostMax
            fixed_recip_join();
            fixed_field(e);
            if (set.polarization_type == MPID_MUTUAL) {
                mutual_mixed_start(e);
                cg_begin<float, float>(e, b32.p, x32.p, r32.p, p32.p, q32.p, inner_target(), K);
                for (int i = 0; i < K; ++i) cg_iteration<float, float>(e, x32.p, r32.p, p32.p, q32.p, inner_target(), K, i == 0);
                op_copy(hostDone + 256, iter.p, sizeof(int), cudaMemcpyDeviceToHost, st);
                launch_check(e, *ed);  // the FP64 residual to refHost, beside the force/energy phase
                finish(e, ptMuF.p, ptEF.p, ptGF.p);
                op_wait(st, evRefDone);
            } else {
                solve_dipoles(e, ptMuF.p, ptEF.p, ptGF.p);
                finish(e, ptMuF.p, ptEF.p, ptGF.p);
            }
            launch<k_forces_out>(nblk(n, 128), 128, 0, st, n, npad, e.rank.p, forceFx.p, forcesOut.p);
        } else {
            Engine<double>& e = *ed;
            sort_and_tiles();
            prepare_engine(e, true);
            fixed_recip_fork(e);  // beside the list build
            launch_lists(e, false);
            fixed_recip_join();
            fixed_field(e);
            if (set.polarization_type == MPID_MUTUAL) {
                cg_begin<double, double>(e, e.SE.p, y64.p, r64.p, p64.p, q64.p, set.mutual_eps, K);
                for (int i = 0; i < K; ++i)
                    cg_iteration<double, double>(e, y64.p, r64.p, p64.p, q64.p, set.mutual_eps, K, i == 0);
                op_copy(hostDone + 256, iter.p, sizeof(int), cudaMemcpyDeviceToHost, st);
                op_copy(hostSc, sc.p, 8 * sizeof(double), cudaMemcpyDeviceToHost, st);
                launch<k_mu_from_y<double, double>>(nblk(npad, 128), 128, 0, st, npad, e.sroot.p, y64.p, e.mu.p);
                finish(e, ptMuD.p, ptED.p, ptGD.p);
            } else {
                solve_dipoles(e, ptMuD.p, ptED.p, ptGD.p);
                finish(e, ptMuD.p, ptED.p, ptGD.p);
            }
            launch<k_forces_out>(nblk(n, 128), 128, 0, st, n, npad, e.rank.p, forceFx.p, forcesOut.p);
        }
        op_copy(hostEparts, energyOut.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, st);
        if (mg || pg) {
            gradPrepared = false;
            if (mg) multipole_gradient_launches();
            if (pg) polarization_gradient_launches();
        }
        CUDA_CHECK(cudaGetLastError());
    }

    // The context's batch graph for the current list shape, box and solver length,
    // captured when it changed; returns true if it was captured now.
    bool ensure_batch_graph(bool mg, bool pg) {
        if (mg || pg) gradient_buffers(mg, pg);  // allocations before the key and the capture
        if (!hostEparts) CUDA_CHECK(cudaMallocHost(&hostEparts, 3 * sizeof(double)));
        const int K = batch_iterations();
        std::vector<long long> key = graph_key(kSegFull);
        const long long more[] = {K, mg ? 1 : 0, pg ? 1 : 0};
        key_put(key, more, sizeof more);
        if (full.graph && full.key == key) return false;
        full.destroy();
        cudaStream_t st = stream;
        const bool wasActive = graphsActive;
        graphsActive = false;  // the body launches directly into this capture
        timer.off = true;
        const long long l0 = t_launches, c0 = t_library_calls;
        cudaGraph_t graph = nullptr;
        CUDA_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            batch_body(mg, pg, K);
        } catch (...) {
            cudaStreamEndCapture(st, &graph);
            if (graph) cudaGraphDestroy(graph);
            (void) cudaGetLastError();
            timer.off = false;
            graphsActive = wasActive;
            t_launches = l0;
            t_library_calls = c0;
            throw;
        }
        const cudaError_t ce = cudaStreamEndCapture(st, &graph);
        timer.off = false;
        graphsActive = wasActive;
        full.nodes = t_launches - l0;
        full.library = t_library_calls - c0;
        t_launches = l0;
        t_library_calls = c0;
        CUDA_CHECK(ce);
        full.graph = graph;
        full.key = key;
        full.K = K;
        full.generation = ++graphClock;
        ++stats.graph_captures;
        return true;
    }

    // The context's evaluation recorded for a fused multi-box launch (the operations of
    // batch_body in issue order, nothing issued), re-recorded when its shape changed;
    // returns true if it was recorded now.  K: the CG iterations of the recording (the
    // largest of the batch's boxes, so that every box issues the same sequence).
    OpRecorder rec;
    std::vector<long long> recKey;
    unsigned long long recGeneration = 0;
    bool ensure_recording(bool mg, bool pg, int K) {
        if (mg || pg) gradient_buffers(mg, pg);
        if (!hostEparts) CUDA_CHECK(cudaMallocHost(&hostEparts, 3 * sizeof(double)));
        std::vector<long long> key = graph_key(kSegFull);
        const long long more[] = {K, mg ? 1 : 0, pg ? 1 : 0};
        key_put(key, more, sizeof more);
        if (!rec.ops.empty() && recKey == key) return false;
        rec.ops.clear();
        recKey.clear();
        const bool wasActive = graphsActive;
        graphsActive = false;
        timer.off = true;
        OpRecorder* prev = t_recorder;
        t_recorder = &rec;
        try {
            batch_body(mg, pg, K);
        } catch (...) {
            t_recorder = prev;
            timer.off = false;
            graphsActive = wasActive;
            rec.ops.clear();
            throw;
        }
        t_recorder = prev;
        timer.off = false;
        graphsActive = wasActive;
        recKey = key;
        recGeneration = ++graphClock;
        return true;
    }
    // CG iterations a batch evaluation of this context runs (the last solve's plus one).
    int batch_iterations() const {
        return set.polarization_type == MPID_MUTUAL ? std::max(1, std::min(set.max_iter, predictedIters + 1)) : 0;
    }

    // After a batch launch: whether this context's results stand (its lists fitted the
    // capacities and work items the graph was built with, its solver converged).  Also
    // fills the statistics of the evaluation.
    bool batch_ok(long long launches, long long library) {
        const int mTiles = hostMax[0], mTotal = hostMax[1], mL = hostMax[2], mS = hostMax[3];
        lastTiles = mTiles;
        lastMaxList = mTotal;
        stats.max_neighbours = mTotal;
        if (mTiles > tcap || mTotal > cap) return false;
        if ((mL + chunk - 1) / chunk > nchunksL || (mS + chunk - 1) / chunk > nchunksS) return false;
        stats.solver_iterations = 0;
        stats.refinement_steps = 0;
        stats.solver_residual = 0.0;
        if (set.polarization_type == MPID_MUTUAL) {
            const int used = hostDone[256];
            stats.solver_iterations = used;
            if (mixed) {
                const double metric = 48.033324 * std::sqrt(*refHost / n);
                stats.refinement_steps = 1;
                stats.solver_residual = metric;
                if (!(metric < set.mutual_eps)) return false;
            } else {
                stats.solver_residual = hostSc[6];
                if (!(hostSc[6] < set.mutual_eps)) return false;
            }
            predictedIters = used;
        } else if (set.polarization_type == MPID_EXTRAPOLATED) {
            stats.solver_iterations = set.n_extrap - 1;
        }
        stats.energy_parts[0] = hostEparts[0];
        stats.energy_parts[1] = hostEparts[1];
        stats.energy_parts[2] = hostEparts[2];
        stats.kernel_launches = (int) launches;
        stats.library_calls = (int) library;
        stats.graph_replays = 1;
        for (int k = 0; k < ST_COUNT; ++k) {
            stats.ms_stage[k] = 0.0;
            stats.stage_launches[k] = 0;
        }
        stats.ms_total = 0.0;
        evaluated = true;
        gradPrepared = true;  // the graph ran the gradient passes' preparation
        return true;
    }

    // Evaluation with the neighbour lists and per-task energies in `scratch` (the static
    // array above, kNoAllocBytes); allocates nothing and never grows a buffer.
    double evaluate_device_noalloc(const double* d_pos, const double* hbox, double* d_forces, double* d_energy,
                                   void* scratch) {
        if (!usePme)
            throw Error(MPID_ERR_INVALID, "mpid_evaluate_device_noalloc supports PME only (the no-cutoff set-up "
                                          "stages the sort order through host memory)");
        size_t capUse = (kNoAllocListEntries / (size_t) npad) / chunk * chunk;
        const size_t perTile = kNoAllocTasks / (size_t) ntiles;  // work items per tile the array holds
        capUse = std::min(capUse, perTile >= 2 ? (perTile - 2) * chunk : 0);
        if (capUse < (size_t) chunk)
            throw Error(MPID_ERR_INVALID, "mpid_evaluate_device_noalloc: " + std::to_string(n) +
                                              " atoms do not fit the static scratch (at most " +
                                              std::to_string(kNoAllocListEntries / chunk) + " atoms)");
        // Point the list and task-energy buffers at the scratch for this call only.
        struct Redirect {
            Context& c;
            unsigned* listP; size_t listN;
            double* enP; size_t enN;
            int cap; long long entries;
            ~Redirect() {
                c.list.p = listP; c.list.n = listN;
                c.energyBlocks.p = enP; c.energyBlocks.n = enN;
                c.cap = cap; c.listEntries = entries;
                c.growForbidden = false;
            }
        } guard{*this, list.p, list.n, energyBlocks.p, energyBlocks.n, cap, listEntries};
        list.p = (unsigned*) scratch;
        list.n = (size_t) npad * capUse;
        energyBlocks.p = (double*) ((char*) scratch + kNoAllocListEntries * 4);
        energyBlocks.n = kNoAllocTasks;
        cap = (int) capUse;
        listEntries = (long long) list.n;
        growForbidden = true;
        return evaluate_device(d_pos, hbox, d_forces, d_energy);
    }

    // Mass-weighted centre, then the 13 system moments of the last evaluation
    // (MPIDReferenceForce.cpp:2349-2462; Debye and Debye-A units as the reference).
    void system_moments(const double* hostMasses, double* out13) {
        if (!evaluated) throw Error(MPID_ERR_STATE, "no evaluation has been run");
        cudaStream_t st = stream;
        masses.alloc(n);
        CUDA_CHECK(cudaMemcpyAsync(masses.p, hostMasses, n * 8, cudaMemcpyHostToDevice, st));
        const int nb = nblk(n, 256);
        momentPartial.alloc((size_t) 16 * nb);
        momentRed.alloc(16);
        const int* rk = mixed ? ef->rank.p : ed->rank.p;
        for (int pass = 0; pass < 2; ++pass) {
            if (mixed)
                launch<k_moment_partials<float>>(nb, 256, 0, st, n, npad, pass, (const double*) pos.p,
                       (const double*) masses.p, rk, (const double*) mom64.p, (const float*) ef->mu.p,
                       (const double*) momentRed.p, momentPartial.p);
            else
                launch<k_moment_partials<double>>(nb, 256, 0, st, n, npad, pass, (const double*) pos.p,
                       (const double*) masses.p, rk, (const double*) mom64.p, (const double*) ed->mu.p,
                       (const double*) momentRed.p, momentPartial.p);
            launch<k_reduce_partials>(1, 1024, 0, st, nb, pass == 0 ? 4 : 16, (const double*) momentPartial.p,
                   momentRed.p, (const int*) nullptr);
        }
        double v[16];
        CUDA_CHECK(cudaMemcpyAsync(v, momentRed.p, 16 * 8, cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
        const double debye = 4.80321;
        const double qave = (v[4] + v[7] + v[9]) / 3.0;
        double m[13];
        m[0] = v[0];
        for (int k = 0; k < 3; ++k) m[1 + k] = v[1 + k] * 10.0 * debye;
        m[4] = 0.5 * (v[4] - qave) + v[10];
        m[5] = 0.5 * v[5] + v[11];
        m[6] = 0.5 * v[6] + v[12];
        m[8] = 0.5 * (v[7] - qave) + v[13];
        m[9] = 0.5 * v[8] + v[14];
        m[12] = 0.5 * (v[9] - qave) + v[15];
        m[7] = m[5];
        m[10] = m[6];
        m[11] = m[9];
        for (int k = 4; k < 13; ++k) m[k] *= 100.0 * 3.0 * debye;
        std::memcpy(out13, m, sizeof(m));
    }

    // Potential (kJ/mol/e) of the last evaluation's multipoles and induced dipoles at
    // ngrid points (MPIDReferenceForce.cpp:2464-2528).
    void electrostatic_potential(const double* hostGrid, int ngrid, double* out) {
        if (!evaluated) throw Error(MPID_ERR_STATE, "no evaluation has been run");
        if (ngrid < 0) throw Error(MPID_ERR_INVALID, "negative number of grid points");
        if (ngrid == 0) return;
        cudaStream_t st = stream;
        gridPts.alloc(3 * (size_t) ngrid);
        gridOut.alloc(ngrid);
        CUDA_CHECK(cudaMemcpyAsync(gridPts.p, hostGrid, 3 * (size_t) ngrid * 8, cudaMemcpyHostToDevice, st));
        if (mixed)
            launch<k_potential_grid<float>>(nblk(ngrid, 128), 128, 0, st, n, npad, ngrid, (const double*) gridPts.p,
                   (const double*) wpos.p, (const int*) ef->rank.p, (const double*) mom64.p, (const float*) ef->mu.p, box,
                   usePme ? 1 : 0, gridOut.p);
        else
            launch<k_potential_grid<double>>(nblk(ngrid, 128), 128, 0, st, n, npad, ngrid, (const double*) gridPts.p,
                   (const double*) wpos.p, (const int*) ed->rank.p, (const double*) mom64.p, (const double*) ed->mu.p,
                   box, usePme ? 1 : 0, gridOut.p);
        CUDA_CHECK(cudaMemcpyAsync(out, gridOut.p, (size_t) ngrid * 8, cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaStreamSynchronize(st));
    }

    // The gradient passes run in FP64 on both paths.  On the mixed path their inputs are
    // prepared once per evaluation in the FP64 engine: the atoms (lab moments, offsets,
    // B-splines), the mixed solve's induced dipoles (the refined FP64 dipoles for Mutual,
    // the FP32 ones widened otherwise) and the FP64 reciprocal potentials of the
    // permanent multipoles and of those dipoles.  The per-type sums of a fitting
    // workload cancel strongly, which FP32 pair and PME terms would not resolve.
    Engine<double>& gradient_engine() {
        if (!mixed) return *ed;
        if (gradPrepared) return ed ? *ed : *eg;
        cudaStream_t st = stream;
        // Mutual: the refinement engine, whose dipoles are the refined FP64 ones
        Engine<double>* dp = ed.get();
        if (!dp) {
            if (!eg) {
                eg.reset(new Engine<double>());
                eg->init(n, npad, usePme, set.pme_order, set.grid, numSMs);
            }
            dp = eg.get();
        }
        Engine<double>& d = *dp;
        prepare_engine(d, true);
        if (dp != ed.get()) {
            const size_t n3 = 3 * (size_t) npad;
            op_memset(d.mu.p, 0, n3 * 8, st);
            launch<k_axpy_to_double<float>>(nblk((long long) n3, 256), 256, 0, st, (int) n3, (const float*) ef->mu.p,
                   d.mu.p);
        }
        if (usePme) {
            fork_pme();
            cudaStream_t ps = pmeStream;
            d.pme.template spread<20>(n, npad, box, d.mf.p, nullptr, ps);
            d.pme.convolve(influence.p, nullptr, ps);
            d.pme.template gather<35>(n, npad, box, d.phiP.p, nullptr, ps);
            launch<k_frac_dipoles<double>>(nblk(npad, 128), 128, 0, ps, npad, box, (const double*) d.mu.p, d.mfd.p,
                   (const int*) nullptr);
            d.pme.template spread<4>(n, npad, box, d.mfd.p, nullptr, ps);
            d.pme.convolve(influence.p, nullptr, ps);
            d.pme.template gather<35>(n, npad, box, d.phiD.p, nullptr, ps);
            join_pme();
        }
        CUDA_CHECK(cudaGetLastError());
        gradPrepared = true;
        return d;
    }

    // Sub-ranges per work item for a gradient launch whose busy items number `items`:
    // enough warps to cover every SM several times (a power of two dividing the chunk).
    int gradient_split(long long items) const {
        int split = 1;
        while (split < chunk && items * split < 16LL * numSMs) split *= 2;
        return split;
    }
    int gradient_blocks(int split) const { return std::max(1, nblk((long long) pair_tasks() * split, kWarpsPerBlock)); }

    // dE/d(molecular-frame polarisability X Y Z, Thole width) of every atom for the last
    // evaluation (Mutual, Direct, Extrapolated).
    void polarization_gradients(double* host, bool wait = true) {
        if (!evaluated) throw Error(MPID_ERR_STATE, "no evaluation has been run");
        gradient_buffers(false, true);
        polarization_gradient_launches();
        CUDA_CHECK(cudaMemcpyAsync(host, polOut.p, (size_t) 4 * n * 8, cudaMemcpyDeviceToHost, stream));
        if (wait) CUDA_CHECK(cudaStreamSynchronize(stream));
    }

    // Device buffers of the gradient passes (allocated before any launch is queued, so
    // that the launches can be captured).
    void gradient_buffers(bool multipole, bool polarization) {
        if (listsInScratch)
            throw Error(MPID_ERR_STATE, "the last evaluation kept its neighbour lists in the allocation-free call's "
                                        "scratch; evaluate with mpid_evaluate_device or a host-buffer call first");
        if (mixed && !ed && !eg) {
            eg.reset(new Engine<double>());
            eg->init(n, npad, usePme, set.pme_order, set.grid, numSMs);
        }
        if (multipole) {
            gradFx.alloc((size_t) 20 * npad);
            gradOut.alloc((size_t) 20 * n);
        }
        if (polarization) {
            polFx.alloc((size_t) 2 * npad);
            polOut.alloc((size_t) 4 * n);
            if (set.polarization_type == MPID_EXTRAPOLATED && mixed) {
                const size_t n3 = 3 * (size_t) npad;
                const int nPT = set.n_extrap;
                gradPtMu.alloc((size_t) nPT * n3);
                gradPtE.alloc((size_t) std::max(nPT - 1, 1) * n3);
                gradEfix.alloc(n3);
            }
        }
    }

    // The polarisation-gradient pass into polOut (launches only).
    void polarization_gradient_launches() {
        Engine<double>& d = gradient_engine();
        cudaStream_t st = stream;
        op_memset(polFx.p, 0, (size_t) 2 * npad * 8, st);
        const int mutual = set.polarization_type == MPID_MUTUAL ? 1 : 0;
        // Extrapolated: the perturbation orders, their fields and the permanent field
        // (FP64 copies of the mixed path's FP32 ones for the FP64 parts)
        OptOrders<float> optF{};
        OptOrders<double> optD{};
        const double* efixD = d.Efix.p;
        const double* ptED = this->ptED.p;
        if (set.polarization_type == MPID_EXTRAPOLATED) {
            const int nPT = set.n_extrap;
            optF.nPT = optD.nPT = nPT;
            for (int i = 0; i < nPT; ++i) {
                double c = 0.0;
                for (int j = i; j < nPT; ++j) c += set.extrap_coeffs[j];
                optF.cbar[i] = optD.cbar[i] = c;
            }
            if (mixed) {
                const size_t n3 = 3 * (size_t) npad;
                op_memset(gradPtMu.p, 0, (size_t) nPT * n3 * 8, st);
                op_memset(gradPtE.p, 0, (size_t) std::max(nPT - 1, 1) * n3 * 8, st);
                op_memset(gradEfix.p, 0, n3 * 8, st);
                launch<k_axpy_to_double<float>>(nblk((long long) nPT * n3, 256), 256, 0, st, (int) (nPT * n3),
                       (const float*) ptMuF.p, gradPtMu.p);
                if (nPT > 1)
                    launch<k_axpy_to_double<float>>(nblk((long long) (nPT - 1) * n3, 256), 256, 0, st,
                           (int) ((nPT - 1) * n3), (const float*) ptEF.p, gradPtE.p);
                launch<k_axpy_to_double<float>>(nblk((long long) n3, 256), 256, 0, st, (int) n3,
                       (const float*) ef->Efix.p, gradEfix.p);
                optF.mu = ptMuF.p;
                optD.mu = gradPtMu.p;
                efixD = gradEfix.p;
                ptED = gradPtE.p;
            } else {
                optD.mu = ptMuD.p;
            }
        }
        const int sL = gradient_split((long long) ntiles * nchunksL), sS = gradient_split((long long) ntiles * nchunksS);
        const int sA = gradient_split(pair_tasks());
        if (mixed && usePme) {
            launch<k_polarization_gradient<float>>(gradient_blocks(sL), 32 * kWarpsPerBlock, 0, st, nbr_list(),
                   ef->arrays(), (const float*) ef->mu.p, mutual, optF, polFx.p, kSegErfc, sL);
            launch<k_polarization_gradient<double>>(gradient_blocks(sS), 32 * kWarpsPerBlock, 0, st, nbr_list(),
                   d.arrays(), (const double*) d.mu.p, mutual, optD, polFx.p, kSegQuad, sS);
        } else {
            launch<k_polarization_gradient<double>>(gradient_blocks(sA), 32 * kWarpsPerBlock, 0, st, nbr_list(),
                   d.arrays(), (const double*) d.mu.p, mutual, optD, polFx.p, kSegAll, sA);
        }
        launch<k_polarization_gradient_finish<double>>(nblk(n, 32), 32, 0, st, n, npad, (const int*) order.p, mol(),
               (const double*) pos.p, (const unsigned long long*) polFx.p, (const double*) d.mu.p, optD, efixD, ptED,
               polOut.p);
        CUDA_CHECK(cudaGetLastError());
    }

    // dE/d(molecular-frame multipole parameters) of every atom for the last evaluation.
    // The real-space sum runs in FP64 except, on the mixed path under PME, over the erfc
    // segment of the lists (alpha r >= 1.5, no excluded pairs), which runs in FP32.  Without
    // a cutoff every pair is bare 1/r, near ones included, and FP32 rank-6 derivative
    // tensors of those cost 1.6e-4 relative (160-atom test system), so all run in FP64.
    void parameter_gradients(double* host, bool wait = true) {
        if (!evaluated) throw Error(MPID_ERR_STATE, "no evaluation has been run");
        gradient_buffers(true, false);
        multipole_gradient_launches();
        CUDA_CHECK(cudaMemcpyAsync(host, gradOut.p, (size_t) 20 * n * 8, cudaMemcpyDeviceToHost, stream));
        if (wait) CUDA_CHECK(cudaStreamSynchronize(stream));
    }

    // The multipole-gradient pass into gradOut (launches only).
    void multipole_gradient_launches() {
        Engine<double>& d = gradient_engine();
        cudaStream_t st = stream;
        op_memset(gradFx.p, 0, (size_t) 20 * npad * 8, st);
        const int sL = gradient_split((long long) ntiles * nchunksL), sS = gradient_split((long long) ntiles * nchunksS);
        const int sA = gradient_split(pair_tasks());
        if (mixed && usePme) {
            launch<k_multipole_gradient<float>>(gradient_blocks(sL), 32 * kWarpsPerBlock, 0, st, nbr_list(),
                   ef->arrays(), (const float*) ef->mu.p, gradFx.p, kSegErfc, sL);
            launch<k_multipole_gradient<double>>(gradient_blocks(sS), 32 * kWarpsPerBlock, 0, st, nbr_list(),
                   d.arrays(), (const double*) d.mu.p, gradFx.p, kSegQuad, sS);
        } else {
            launch<k_multipole_gradient<double>>(gradient_blocks(sA), 32 * kWarpsPerBlock, 0, st, nbr_list(),
                   d.arrays(), (const double*) d.mu.p, gradFx.p, kSegAll, sA);
        }
        launch<k_gradient_finish<double>>(nblk(n, 32), 32, 0, st, n, npad, box, usePme ? set.ewald_alpha : 0.0,
               usePme ? 1 : 0, (const int*) order.p, mol(), (const double*) pos.p, (const unsigned long long*) gradFx.p,
               (const double*) d.phiP.p, (const double*) d.phiD.p, (const double*) mom64.p, (const double*) d.mu.p,
               gradOut.p);
        CUDA_CHECK(cudaGetLastError());
    }

    // Both gradient passes after an evaluation: with graphs, one captured segment (the
    // FP64 inputs of the pass, then each pass), then the copies to the host.
    void gradients(double* multipoleHost, double* polarizationHost) {
        const bool mg = multipoleHost != nullptr, pg = polarizationHost != nullptr;
        if (!mg && !pg) {
            if (!evaluated) throw Error(MPID_ERR_STATE, "no evaluation has been run");
            return;
        }
        gradients_device(mg, pg);
        if (mg) CUDA_CHECK(cudaMemcpyAsync(multipoleHost, gradOut.p, (size_t) 20 * n * 8, cudaMemcpyDeviceToHost, stream));
        if (pg) CUDA_CHECK(cudaMemcpyAsync(polarizationHost, polOut.p, (size_t) 4 * n * 8, cudaMemcpyDeviceToHost, stream));
    }

    // The gradient passes into gradOut / polOut (device), replayed from a graph.
    void gradients_device(bool mg, bool pg) {
        if (!evaluated) throw Error(MPID_ERR_STATE, "no evaluation has been run");
        if (!mg && !pg) return;
        gradient_buffers(mg, pg);
        const bool prepared = gradPrepared;
        std::vector<long long> key = graph_key(kSegGradients);
        key.push_back((mg ? 1 : 0) | (pg ? 2 : 0) | (prepared ? 4 : 0));
        const long long launches0 = t_launches, library0 = t_library_calls;
        replay(key, [&] {
            if (mg) multipole_gradient_launches();
            if (pg) polarization_gradient_launches();
        });
        // the gradient passes count with the evaluation they belong to
        stats.kernel_launches += (int) (t_launches - launches0);
        stats.library_calls += (int) (t_library_calls - library0);
        gradPrepared = true;  // a replay does not run gradient_engine's host side
    }

    void get_dipoles(int which, double* host) {
        if (!evaluated) throw Error(MPID_ERR_STATE, "no evaluation has been run");
        if (which < 0 || which > 3) throw Error(MPID_ERR_INVALID, "which must be 0, 1, 2 or 3");
        if (which == 3) {  // permanent field: reuse the induced-dipole output path with mom = 0
            if (mixed)
                launch<k_dipoles_out<float>>(nblk(n, 128), 128, 0, stream, n, npad, 0, ef->rank.p, ef->mom.p, ef->Efix.p, forcesOut.p);
            else
                launch<k_dipoles_out<double>>(nblk(n, 128), 128, 0, stream, n, npad, 0, ed->rank.p, ed->mom.p, ed->Efix.p, forcesOut.p);
        } else if (mixed)
            launch<k_dipoles_out<float>>(nblk(n, 128), 128, 0, stream, n, npad, which, ef->rank.p, ef->mom.p, ef->mu.p, forcesOut.p);
        else
            launch<k_dipoles_out<double>>(nblk(n, 128), 128, 0, stream, n, npad, which, ed->rank.p, ed->mom.p, ed->mu.p, forcesOut.p);
        CUDA_CHECK(cudaGetLastError());
        CUDA_CHECK(cudaMemcpyAsync(host, forcesOut.p, 3 * (size_t) n * 8, cudaMemcpyDeviceToHost, stream));
        CUDA_CHECK(cudaStreamSynchronize(stream));
    }
};

// ---------------------------------------------------------------------------
// Fused multi-box evaluation.  Every box of a batch records its evaluation (the same
// sequence of operations for every box; box-specific parameters and launch sizes).
// Operation i of all boxes then becomes one multi-box operation:
//  - a kernel: one k_boxes launch of its body over the blocks of all boxes (one per
//    distinct block shape, and per BoxParams::kBoxes boxes);
//  - a fill or copy: one k_fill_bytes / k_copy_bytes launch over all boxes;
//  - an FFT: the boxes' grids are gathered into one array per grid size, transformed
//    by one batched cuFFT plan (cufftPlanMany) per size, and scattered back.
// The sequence is captured once as one CUDA graph and replayed while no box's recording
// changes, with the boxes' stream structure (lanes, below): a box's reciprocal-space
// chain runs beside its real-space kernels as in a single-box evaluation.
template <auto F, class... A>
static std::unique_ptr<RecKernel> make_rec(dim3 grid, dim3 block, size_t smem, A&&... a) {
    std::unique_ptr<RecKernelOf<F>> r(new RecKernelOf<F>());
    r->grid = grid;
    r->block = block;
    r->smem = smem;
    r->args = Launcher<F, typename KTraits<F>::Args>::pack(std::forward<A>(a)...);
    return r;
}

struct FusedBatch {
    std::vector<unsigned long long> key;  // per box: context id, recording generation
    cudaGraphExec_t exec = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t evStart = nullptr, evStop = nullptr;
    int device = -1;
    long long launches = 0, library = 0;  // per replay
    std::map<std::vector<int>, cufftHandle> plans;  // (bytes per real, forward, nx, ny, nz, count)
    // gather (input) and result (output) arrays of the batched FFTs, per lane (lanes may
    // transform at the same time); the plans are per lane too
    std::map<int, DBuf<unsigned char>> arenaIn, arenaOut;
    // Streams and events on which the FFT groups of one operation (one per grid size)
    // run side by side: each is only a few small cuFFT kernels.
    std::vector<cudaStream_t> fftStreams;
    std::vector<cudaEvent_t> fftEvents;  // [0] the fork, then one join per stream
    // The lanes beyond the first (the boxes' side streams) and the events between them.
    std::vector<cudaStream_t> laneStreams;
    std::vector<cudaEvent_t> laneEvents;
    // Pinned staging of the host arrays, one DMA copy each way at the graph's start and
    // end, scattered to and gathered from the boxes' device buffers by one launch each:
    // per box, positions and incoming forces (6n doubles at inOff), forces, multipole and
    // polarisation gradients (3n + 20n + 4n at outOff, the gradients when requested).
    double* hostIn = nullptr;
    double* hostOut = nullptr;
    size_t hostInCount = 0, hostOutCount = 0;
    DBuf<double> devIn, devOut;  // device copies of the staging (one DMA copy each way)
    // The recorded copies into the boxes' pinned host variables (list maxima, solver
    // state, FP64 residual, energies) land in devOut too, at `offset` doubles, and reach
    // their host destination after the launch (in recording order): kernels writing the
    // host memory directly would cost a host-memory round trip per box and operation.
    struct HostCopy {
        void* dst;
        size_t offset, bytes;
    };
    std::vector<HostCopy> hostCopies;
    std::vector<size_t> inOff, outOff;
    void reset_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        key.clear();
    }
    void release() {
        reset_graph();
        for (auto& kv : plans) cufftDestroy(kv.second);
        plans.clear();
        arenaIn.clear();
        arenaOut.clear();
        devIn.free();
        devOut.free();
        if (hostIn) cudaFreeHost(hostIn);
        if (hostOut) cudaFreeHost(hostOut);
        hostIn = hostOut = nullptr;
        hostInCount = hostOutCount = 0;
        for (cudaStream_t q : fftStreams) cudaStreamDestroy(q);
        for (cudaEvent_t ev : fftEvents) cudaEventDestroy(ev);
        fftStreams.clear();
        fftEvents.clear();
        for (cudaStream_t q : laneStreams) cudaStreamDestroy(q);
        for (cudaEvent_t ev : laneEvents) cudaEventDestroy(ev);
        laneStreams.clear();
        laneEvents.clear();
        if (evStart) cudaEventDestroy(evStart);
        if (evStop) cudaEventDestroy(evStop);
        evStart = evStop = nullptr;
        if (stream) cudaStreamDestroy(stream);
        stream = nullptr;
    }
};

// One launch copying every (dst, src, bytes) of `copies` (k_copy_bytes, one entry per copy).
static void copy_group(const std::vector<std::tuple<void*, const void*, size_t>>& copies, cudaStream_t st) {
    if (copies.empty()) return;
    std::vector<std::unique_ptr<RecKernel>> tmp;
    std::vector<const RecKernel*> grp;
    for (const auto& c : copies) {
        const size_t bytes = std::get<2>(c);
        tmp.push_back(make_rec<k_copy_bytes>(std::max(1, std::min(64, nblk((long long) (bytes / 16), 256))), 256, 0,
                                             (unsigned char*) std::get<0>(c), (const unsigned char*) std::get<1>(c), bytes));
        grp.push_back(tmp.back().get());
    }
    grp[0]->launch_group(grp, st);
}

static size_t fft_bytes(const RecOp& op, bool input) {
    const size_t G = (size_t) op.fftDims[0] * op.fftDims[1] * op.fftDims[2];
    const size_t Gh = (size_t) op.fftDims[0] * op.fftDims[1] * (op.fftDims[2] / 2 + 1);
    const bool realSide = (op.fftForward != 0) == input;
    return realSide ? G * op.fftPrec : Gh * 2 * op.fftPrec;
}
static size_t align256(size_t b) { return (b + 255) & ~(size_t) 255; }

// The boxes of an FFT operation grouped by grid size, each with its offsets in the
// gather (input) and result (output) arrays; returns the bytes of both.
struct FftSlot {
    int box;
    size_t in, out;
};
static std::map<std::vector<int>, std::vector<FftSlot>> fft_groups(const std::vector<const RecOp*>& ops, size_t& inBytes,
                                                                   size_t& outBytes) {
    std::map<std::vector<int>, std::vector<FftSlot>> groups;
    for (int b = 0; b < (int) ops.size(); ++b)
        groups[{ops[b]->fftDims[0], ops[b]->fftDims[1], ops[b]->fftDims[2]}].push_back({b, 0, 0});
    inBytes = outBytes = 0;
    for (auto& kv : groups) {
        inBytes = align256(inBytes);
        outBytes = align256(outBytes);
        for (FftSlot& sl : kv.second) {
            sl.in = inBytes;
            sl.out = outBytes;
            inBytes += fft_bytes(*ops[sl.box], true);
            outBytes += fft_bytes(*ops[sl.box], false);
        }
    }
    return groups;
}

static void fused_fft(FusedBatch& fb, const std::vector<const RecOp*>& ops, cudaStream_t st, int lane) {
    DBuf<unsigned char>& arenaIn = fb.arenaIn[lane];
    DBuf<unsigned char>& arenaOut = fb.arenaOut[lane];
    size_t inBytes, outBytes;
    const auto groups = fft_groups(ops, inBytes, outBytes);
    const RecOp& a = *ops[0];
    std::vector<std::unique_ptr<RecKernel>> gather, scatter;
    for (const auto& kv : groups)
        for (const FftSlot& sl : kv.second) {
            const RecOp& op = *ops[sl.box];
            const size_t bi = fft_bytes(op, true), bo = fft_bytes(op, false);
            gather.push_back(make_rec<k_copy_bytes>(std::max(1, std::min(64, nblk((long long) (bi / 16), 256))), 256, 0,
                                                    arenaIn.p + sl.in, (const unsigned char*) op.src, bi));
            scatter.push_back(make_rec<k_copy_bytes>(std::max(1, std::min(64, nblk((long long) (bo / 16), 256))), 256, 0,
                                                     (unsigned char*) op.dst, (const unsigned char*) arenaOut.p + sl.out, bo));
        }
    std::vector<const RecKernel*> g(gather.size()), s(scatter.size());
    for (size_t i = 0; i < gather.size(); ++i) {
        g[i] = gather[i].get();
        s[i] = scatter[i].get();
    }
    g[0]->launch_group(g, st);
    // the size groups side by side, each on its own stream, joined back into st
    const int ng = (int) groups.size();
    if (ng > 1) {
        if ((int) fb.fftStreams.size() < ng || (int) fb.fftEvents.size() < ng + 1)
            throw Error(MPID_ERR_STATE, "fused batch: FFT streams not prepared");
        CUDA_CHECK(cudaEventRecord(fb.fftEvents[0], st));
        for (int q = 0; q < ng; ++q) CUDA_CHECK(cudaStreamWaitEvent(fb.fftStreams[q], fb.fftEvents[0], 0));
    }
    int q = 0;
    for (const auto& kv : groups) {
        const std::vector<int> pk = {a.fftPrec, a.fftForward, kv.first[0], kv.first[1], kv.first[2], (int) kv.second.size(),
                                     lane};
        cufftHandle h = fb.plans.at(pk);
        cudaStream_t gs = ng > 1 ? fb.fftStreams[q] : st;
        ++q;
        CUFFT_CHECK(cufftSetStream(h, gs));
        void* in = arenaIn.p + kv.second[0].in;
        void* out = arenaOut.p + kv.second[0].out;
        if (a.fftPrec == 4 && a.fftForward)
            CUFFT_CHECK(cufftExecR2C(h, (cufftReal*) in, (cufftComplex*) out));
        else if (a.fftPrec == 4)
            CUFFT_CHECK(cufftExecC2R(h, (cufftComplex*) in, (cufftReal*) out));
        else if (a.fftForward)
            CUFFT_CHECK(cufftExecD2Z(h, (cufftDoubleReal*) in, (cufftDoubleComplex*) out));
        else
            CUFFT_CHECK(cufftExecZ2D(h, (cufftDoubleComplex*) in, (cufftDoubleReal*) out));
        ++t_library_calls;
    }
    if (ng > 1)
        for (int k = 0; k < ng; ++k) {
            CUDA_CHECK(cudaEventRecord(fb.fftEvents[1 + k], fb.fftStreams[k]));
            CUDA_CHECK(cudaStreamWaitEvent(st, fb.fftEvents[1 + k], 0));
        }
    s[0]->launch_group(s, st);
}

// Checks that the boxes' recordings match operation by operation, prepares the FFT
// plans and arrays, and captures the fused sequence as fb's graph.
// outMg / outPg: copy every box's per-atom multipole / polarisation gradients to the
// staging; typeSums: reduce them per atom type on the device instead (k_type_sums).
static void fused_build(FusedBatch& fb, const std::vector<Context*>& boxes, bool outMg, bool outPg, bool typeSums) {
    const size_t L = boxes[0]->rec.ops.size();
    for (Context* c : boxes)
        if (c->rec.ops.size() != L)
            throw Error(MPID_ERR_INVALID, "fused batch: the boxes' evaluations differ in their operations");
    struct FftInfo {
        size_t i, in, out;
        std::vector<std::vector<int>> keys;
    };
    std::vector<FftInfo> fftInfo;
    std::vector<const RecOp*> ops(boxes.size());
    for (size_t i = 0; i < L; ++i) {
        const RecOp& a = boxes[0]->rec.ops[i];
        for (size_t b = 0; b < boxes.size(); ++b) {
            const RecOp& o = boxes[b]->rec.ops[i];
            ops[b] = &o;
            const bool same = o.kind == a.kind && (a.kind != RecOp::KERNEL || o.k->body() == a.k->body()) &&
                              (a.kind != RecOp::FFT || (o.fftPrec == a.fftPrec && o.fftForward == a.fftForward));
            if (!same) throw Error(MPID_ERR_INVALID, "fused batch: the boxes' evaluations differ in their operations");
        }
        if (a.kind == RecOp::FFT) {
            FftInfo fi{i, 0, 0, {}};
            for (const auto& kv : fft_groups(ops, fi.in, fi.out))
                fi.keys.push_back({a.fftPrec, a.fftForward, kv.first[0], kv.first[1], kv.first[2], (int) kv.second.size()});
            fftInfo.push_back(std::move(fi));
        }
    }
    // Lanes: each box's streams and events numbered by first use.  Boxes that follow the
    // same code path number them alike, and the fused graph then runs lane l's
    // operations on stream l with the recorded event dependencies between lanes (the
    // reciprocal-space chain beside the real-space kernels, the FP64 residual check
    // beside the force phase).  Otherwise one lane, and the events are dropped.
    std::vector<int> laneOf(L, 0), slotOf(L, -1);
    size_t nLanes = 1, nSlots = 0;
    bool lanesOk = true;
    for (size_t b = 0; b < boxes.size() && lanesOk; ++b) {
        std::map<cudaStream_t, int> lane;
        std::map<cudaEvent_t, int> slot;
        lane[boxes[b]->rec.ops[0].stream] = 0;
        for (size_t i = 0; i < L; ++i) {
            const RecOp& o = boxes[b]->rec.ops[i];
            auto it = lane.find(o.stream);
            int l;
            if (it == lane.end()) {
                l = (int) lane.size();
                lane[o.stream] = l;
            } else {
                l = it->second;
            }
            int e = -1;
            if (o.kind == RecOp::EV_RECORD || o.kind == RecOp::EV_WAIT) {
                auto jt = slot.find(o.event);
                if (jt == slot.end()) {
                    e = (int) slot.size();
                    slot[o.event] = e;
                } else {
                    e = jt->second;
                }
            }
            if (b == 0) {
                laneOf[i] = l;
                slotOf[i] = e;
            } else if (laneOf[i] != l || slotOf[i] != e) {
                lanesOk = false;
                break;
            }
        }
        if (b == 0) {
            nLanes = lane.size();
            nSlots = slot.size();
        }
    }
    if (!lanesOk) {
        std::fill(laneOf.begin(), laneOf.end(), 0);
        nLanes = 1;
    }
    while (fb.laneStreams.size() + 1 < nLanes) {
        cudaStream_t q;
        CUDA_CHECK(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
        fb.laneStreams.push_back(q);
    }
    while (fb.laneEvents.size() < nSlots + nLanes + 1) {
        cudaEvent_t ev;
        CUDA_CHECK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        fb.laneEvents.push_back(ev);
    }
    fb.reset_graph();
    // pinned staging of the inputs and outputs
    size_t nIn = 0, nOut = 0;
    fb.inOff.assign(boxes.size(), 0);
    fb.outOff.assign(boxes.size(), 0);
    for (size_t b = 0; b < boxes.size(); ++b) {
        const size_t n = (size_t) boxes[b]->n;
        fb.inOff[b] = nIn;
        fb.outOff[b] = nOut;
        nIn += (6 * n + 1) & ~(size_t) 1;  // 16-byte aligned starts
        nOut += (3 * n + (outMg ? 20 * n : 0) + (outPg ? 4 * n : 0) + (typeSums ? 24 * (size_t) boxes[b]->ntypes : 0) + 1) &
                ~(size_t) 1;
    }
    if (nIn > fb.hostInCount) {
        if (fb.hostIn) cudaFreeHost(fb.hostIn);
        fb.hostIn = nullptr;
        fb.hostInCount = 0;
        CUDA_CHECK(cudaMallocHost(&fb.hostIn, nIn * sizeof(double)));
        fb.hostInCount = nIn;
    }
    // device slots of the copies into host memory
    fb.hostCopies.clear();
    for (size_t i = 0; i < L; ++i)
        for (Context* c : boxes) {
            const RecOp& o = c->rec.ops[i];
            if (o.kind != RecOp::COPY) continue;
            cudaPointerAttributes at{};
            CUDA_CHECK(cudaPointerGetAttributes(&at, o.dst));
            if (at.type != cudaMemoryTypeHost) continue;
            fb.hostCopies.push_back({o.dst, nOut, o.bytes});
            nOut += ((o.bytes + 15) / 16) * 2;
        }
    if (nOut > fb.hostOutCount) {
        if (fb.hostOut) cudaFreeHost(fb.hostOut);
        fb.hostOut = nullptr;
        fb.hostOutCount = 0;
        CUDA_CHECK(cudaMallocHost(&fb.hostOut, nOut * sizeof(double)));
        fb.hostOutCount = nOut;
    }
    if (!fb.evStart) CUDA_CHECK(cudaEventCreate(&fb.evStart));
    if (!fb.evStop) CUDA_CHECK(cudaEventCreate(&fb.evStop));
    std::vector<std::tuple<void*, const void*, size_t>> copyIn, copyOut;
    std::vector<std::unique_ptr<RecKernel>> sums;  // per-type sums of each box's gradients
    fb.devIn.alloc(nIn);
    fb.devOut.alloc(nOut);
    for (size_t b = 0; b < boxes.size(); ++b) {
        Context& c = *boxes[b];
        const size_t n = (size_t) c.n;
        const double* in = fb.devIn.p + fb.inOff[b];
        double* out = fb.devOut.p + fb.outOff[b];
        copyIn.emplace_back(c.pos.p, in, 3 * n * 8);
        copyIn.emplace_back(c.forcesOut.p, in + 3 * n, 3 * n * 8);
        copyOut.emplace_back(out, c.forcesOut.p, 3 * n * 8);
        if (outMg) copyOut.emplace_back(out + 3 * n, c.gradOut.p, 20 * n * 8);
        if (outPg) copyOut.emplace_back(out + 3 * n + (outMg ? 20 * n : 0), c.polOut.p, 4 * n * 8);
        if (typeSums)
            sums.push_back(make_rec<k_type_sums>(1, 24 * 32, 0, c.n, (const int*) c.atomTypes.p, c.ntypes,
                                                 (const double*) c.gradOut.p, (const double*) c.polOut.p,
                                                 out + 3 * n + (outMg ? 20 * n : 0) + (outPg ? 4 * n : 0)));
    }
    std::map<int, size_t> inMax, outMax;
    std::vector<std::vector<int>> planKeys;
    for (FftInfo& fi : fftInfo) {
        const int lane = laneOf[fi.i];
        inMax[lane] = std::max(inMax[lane], fi.in);
        outMax[lane] = std::max(outMax[lane], fi.out);
        for (auto& k : fi.keys) {
            k.push_back(lane);
            planKeys.push_back(k);
        }
    }
    for (const auto& kv : inMax) fb.arenaIn[kv.first].alloc(kv.second);
    for (const auto& kv : outMax) fb.arenaOut[kv.first].alloc(kv.second);
    size_t maxGroups = 1;
    for (size_t i = 0; i < L; ++i) {
        if (boxes[0]->rec.ops[i].kind != RecOp::FFT) continue;
        std::set<std::vector<int>> dims;
        for (Context* c : boxes) {
            const RecOp& o = c->rec.ops[i];
            dims.insert({o.fftDims[0], o.fftDims[1], o.fftDims[2]});
        }
        maxGroups = std::max(maxGroups, dims.size());
    }
    while (fb.fftStreams.size() < maxGroups) {
        cudaStream_t q;
        CUDA_CHECK(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
        fb.fftStreams.push_back(q);
    }
    while (fb.fftEvents.size() < maxGroups + 1) {
        cudaEvent_t ev;
        CUDA_CHECK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        fb.fftEvents.push_back(ev);
    }
    for (const auto& pk : planKeys) {
        if (fb.plans.count(pk)) continue;
        int dims[3] = {pk[2], pk[3], pk[4]};
        const cufftType t = pk[0] == 4 ? (pk[1] ? CUFFT_R2C : CUFFT_C2R) : (pk[1] ? CUFFT_D2Z : CUFFT_Z2D);
        cufftHandle h;
        CUFFT_CHECK(cufftPlanMany(&h, 3, dims, nullptr, 1, 0, nullptr, 1, 0, t, pk[5]));
        fb.plans[pk] = h;
    }
    cudaStream_t st = fb.stream;
    const long long l0 = t_launches, c0 = t_library_calls;
    cudaGraph_t graph = nullptr;
    CUDA_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    size_t nextHost = 0;  // the next host-destination copy (same order as the slots)
    try {
        CUDA_CHECK(cudaMemcpyAsync(fb.devIn.p, fb.hostIn, nIn * sizeof(double), cudaMemcpyHostToDevice, st));
        copy_group(copyIn, st);
        // lane l on stream lanes[l]; a lane joins the capture at its first operation (an
        // event wait, or else a fork from lane 0 at that point)
        std::vector<cudaStream_t> lanes(nLanes, st);
        for (size_t l = 1; l < nLanes; ++l) lanes[l] = fb.laneStreams[l - 1];
        std::vector<char> joined(nLanes, 0);
        joined[0] = 1;
        cudaEvent_t* slotEv = fb.laneEvents.data();
        cudaEvent_t* laneEv = fb.laneEvents.data() + nSlots;  // forks and final joins
        for (size_t i = 0; i < L; ++i) {
            for (size_t b = 0; b < boxes.size(); ++b) ops[b] = &boxes[b]->rec.ops[i];
            const RecOp& a = *ops[0];
            const int l = laneOf[i];
            cudaStream_t ls = lanes[l];
            if (!joined[l] && !(lanesOk && a.kind == RecOp::EV_WAIT)) {
                CUDA_CHECK(cudaEventRecord(laneEv[nLanes], st));
                CUDA_CHECK(cudaStreamWaitEvent(ls, laneEv[nLanes], 0));
            }
            joined[l] = 1;
            if (a.kind == RecOp::EV_RECORD || a.kind == RecOp::EV_WAIT) {
                if (!lanesOk) continue;
                if (a.kind == RecOp::EV_RECORD)
                    CUDA_CHECK(cudaEventRecord(slotEv[slotOf[i]], ls));
                else
                    CUDA_CHECK(cudaStreamWaitEvent(ls, slotEv[slotOf[i]], 0));
            } else if (a.kind == RecOp::KERNEL) {
                std::map<std::vector<unsigned>, std::vector<const RecKernel*>> byBlock;
                for (const RecOp* o : ops) byBlock[{o->k->block.x, o->k->block.y, o->k->block.z}].push_back(o->k.get());
                for (const auto& kv : byBlock) kv.second[0]->launch_group(kv.second, ls);
            } else if (a.kind == RecOp::FFT) {
                fused_fft(fb, ops, ls, l);
            } else {
                std::vector<std::unique_ptr<RecKernel>> tmp;
                std::vector<const RecKernel*> grp;
                for (const RecOp* o : ops) {
                    const int blocks = std::max(1, std::min(64, nblk((long long) (o->bytes / 16), 256)));
                    if (o->kind == RecOp::FILL) {
                        tmp.push_back(make_rec<k_fill_bytes>(blocks, 256, 0, (unsigned char*) o->dst, o->value, o->bytes));
                    } else {
                        unsigned char* dst = (unsigned char*) o->dst;
                        if (nextHost < fb.hostCopies.size() && fb.hostCopies[nextHost].dst == o->dst)
                            dst = (unsigned char*) (fb.devOut.p + fb.hostCopies[nextHost++].offset);
                        tmp.push_back(make_rec<k_copy_bytes>(blocks, 256, 0, dst, (const unsigned char*) o->src, o->bytes));
                    }
                    grp.push_back(tmp.back().get());
                }
                grp[0]->launch_group(grp, ls);
            }
        }
        for (size_t l = 1; l < nLanes; ++l)
            if (joined[l]) {
                CUDA_CHECK(cudaEventRecord(laneEv[l], lanes[l]));
                CUDA_CHECK(cudaStreamWaitEvent(st, laneEv[l], 0));
            }
        if (!sums.empty()) {
            std::vector<const RecKernel*> grp;
            for (const auto& r : sums) grp.push_back(r.get());
            grp[0]->launch_group(grp, st);
        }
        copy_group(copyOut, st);
        CUDA_CHECK(cudaMemcpyAsync(fb.hostOut, fb.devOut.p, nOut * sizeof(double), cudaMemcpyDeviceToHost, st));
        CUDA_CHECK(cudaGetLastError());
        if (nextHost != fb.hostCopies.size()) throw Error(MPID_ERR_STATE, "fused batch: host copies out of order");
    } catch (...) {
        cudaStreamEndCapture(st, &graph);
        if (graph) cudaGraphDestroy(graph);
        (void) cudaGetLastError();
        t_launches = l0;
        t_library_calls = c0;
        throw;
    }
    cudaError_t ce = cudaStreamEndCapture(st, &graph);
    fb.launches = t_launches - l0;
    fb.library = t_library_calls - c0;
    t_launches = l0;
    t_library_calls = c0;
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(&fb.exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    CUDA_CHECK(ce);
}

}  // namespace mpid

// ---------------------------------------------------------------------------
// C ABI
using mpid::Context;
using mpid::Error;

static thread_local std::string g_lastError;

#define MPID_API_BEGIN try {
#define MPID_API_END                                   \
    }                                                  \
    catch (const Error& e) {                           \
        g_lastError = e.what();                        \
        return e.code;                                 \
    }                                                  \
    catch (const std::exception& e) {                  \
        g_lastError = e.what();                        \
        return MPID_ERR_CUDA;                          \
    }

struct mpid_context {
    Context ctx;
};

extern "C" {

void mpid_default_settings(mpid_settings* s, int num_atoms) {
    std::memset(s, 0, sizeof(*s));
    s->num_atoms = num_atoms;
    s->nonbonded_method = MPID_NO_CUTOFF;
    s->polarization_type = MPID_EXTRAPOLATED;
    s->cutoff = 1.0;
    s->pme_order = 6;
    s->mutual_eps = 1.0e-5;
    s->max_iter = 60;
    s->n_extrap = 4;
    s->extrap_coeffs[0] = -0.154;
    s->extrap_coeffs[1] = 0.017;
    s->extrap_coeffs[2] = 0.658;
    s->extrap_coeffs[3] = 0.474;
    s->default_thole = 5.0;
    s->scale14 = 1.0;
    s->precision = MPID_PRECISION_MIXED;
}

int mpid_create(const mpid_settings* settings, int device, mpid_context** out) {
    MPID_API_BEGIN
    if (!settings || !out) throw Error(MPID_ERR_INVALID, "null argument");
    mpid::DeviceScope scope(device);
    std::unique_ptr<mpid_context> c(new mpid_context());
    c->ctx.create(*settings, device);
    *out = c.release();
    return MPID_OK;
    MPID_API_END
}

void mpid_destroy(mpid_context* ctx) {
    if (!ctx) return;
    int prev = -1;
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaSetDevice(ctx->ctx.device);
    delete ctx;
    if (prev >= 0) cudaSetDevice(prev);
}

int mpid_set_multipoles(mpid_context* ctx, const double* charge, const double* dipole, const double* quadrupole,
                        const double* octopole, const int* axis_type, const int* atom_z, const int* atom_x,
                        const int* atom_y, const double* thole, const double* polarity) {
    MPID_API_BEGIN
    if (!ctx || !charge || !dipole || !quadrupole || !octopole || !axis_type || !atom_z || !atom_x || !atom_y || !thole ||
        !polarity)
        throw Error(MPID_ERR_INVALID, "null argument");
    mpid::DeviceScope scope(ctx->ctx.device);
    ctx->ctx.set_multipoles(charge, dipole, quadrupole, octopole, axis_type, atom_z, atom_x, atom_y, thole, polarity);
    return MPID_OK;
    MPID_API_END
}

int mpid_set_covalent(mpid_context* ctx, const int* offsets, const int* index) {
    MPID_API_BEGIN
    if (!ctx || !offsets) throw Error(MPID_ERR_INVALID, "null argument");
    mpid::DeviceScope scope(ctx->ctx.device);
    ctx->ctx.set_covalent(offsets, index);
    return MPID_OK;
    MPID_API_END
}

int mpid_set_atom_types(mpid_context* ctx, const int* types, int ntypes) {
    MPID_API_BEGIN
    if (!ctx || (!types && ntypes > 0)) throw Error(MPID_ERR_INVALID, "null argument");
    if (ntypes < 0 || ntypes > mpid::kMaxTypeSums) throw Error(MPID_ERR_INVALID, "ntypes must be in 0..16");
    Context& c = ctx->ctx;
    for (int i = 0; i < c.n && ntypes > 0; ++i)
        if (types[i] < 0 || types[i] >= ntypes) throw Error(MPID_ERR_INVALID, "atom type out of range");
    mpid::DeviceScope scope(c.device);
    if (ntypes > 0) {
        c.atomTypes.alloc(std::max(c.n, 1));
        CUDA_CHECK(cudaMemcpy(c.atomTypes.p, types, (size_t) c.n * sizeof(int), cudaMemcpyHostToDevice));
        c.atomTypesHost.assign(types, types + c.n);
    } else {
        c.atomTypesHost.clear();
    }
    c.ntypes = ntypes;
    return MPID_OK;
    MPID_API_END
}

int mpid_evaluate(mpid_context* ctx, const double* positions, const double* box, double* forces, double* energy) {
    MPID_API_BEGIN
    if (!ctx || !positions || !box || !forces) throw Error(MPID_ERR_INVALID, "null argument");
    Context& c = ctx->ctx;
    mpid::DeviceScope scope(c.device);
    c.stream = c.hostStream;
    const size_t n3 = 3 * (size_t) c.n;
    CUDA_CHECK(cudaMemcpyAsync(c.pos.p, positions, n3 * 8, cudaMemcpyHostToDevice, c.stream));
    CUDA_CHECK(cudaMemcpyAsync(c.forcesOut.p, forces, n3 * 8, cudaMemcpyHostToDevice, c.stream));
    double e = c.evaluate_device(c.pos.p, box, c.forcesOut.p, nullptr);
    CUDA_CHECK(cudaMemcpyAsync(forces, c.forcesOut.p, n3 * 8, cudaMemcpyDeviceToHost, c.stream));
    CUDA_CHECK(cudaStreamSynchronize(c.stream));
    if (energy) *energy = e;
    return MPID_OK;
    MPID_API_END
}

int mpid_evaluate_device(mpid_context* ctx, const double* d_positions, const double* box, double* d_forces,
                         double* d_energy, void* stream) {
    MPID_API_BEGIN
    if (!ctx || !d_positions || !box || !d_forces) throw Error(MPID_ERR_INVALID, "null argument");
    mpid::DeviceScope scope(ctx->ctx.device);
    ctx->ctx.stream = (cudaStream_t) stream;
    ctx->ctx.evaluate_device(d_positions, box, d_forces, d_energy);
    return MPID_OK;
    MPID_API_END
}

// Device address of the static scratch on `device`, looked up once per device with that
// device current (the caller's DeviceScope restores the caller's device afterwards); the
// first call on a device must not run under stream capture.
static std::mutex g_noallocMutex;
static void* g_noallocPtr[mpid::kNoAllocMaxDevices] = {};

static void* noalloc_scratch(int device) {
    if (device < 0 || device >= mpid::kNoAllocMaxDevices) throw Error(MPID_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noallocMutex);
    if (!g_noallocPtr[device]) {
        CUDA_CHECK(cudaSetDevice(device));
        void* p = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (rc != cudaSuccess)
            throw Error(MPID_ERR_CUDA, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(rc));
        g_noallocPtr[device] = p;
    }
    return g_noallocPtr[device];
}

int mpid_evaluate_device_noalloc(mpid_context* ctx, const double* d_positions, const double* box, double* d_forces,
                                 double* d_energy, void* stream) {
    MPID_API_BEGIN
    if (!ctx || !d_positions || !box || !d_forces) throw Error(MPID_ERR_INVALID, "null argument");
    mpid::DeviceScope scope(ctx->ctx.device);
    void* scratch = noalloc_scratch(ctx->ctx.device);
    ctx->ctx.stream = (cudaStream_t) stream;
    ctx->ctx.evaluate_device_noalloc(d_positions, box, d_forces, d_energy, scratch);
    return MPID_OK;
    MPID_API_END
}

// Evaluation at host positions into an internal force buffer (the properties below are
// defined at the positions given, as the reference recomputes the induced dipoles).
static void evaluate_at(Context& c, const double* positions, const double* box) {
    c.stream = c.hostStream;
    const size_t n3 = 3 * (size_t) c.n;
    CUDA_CHECK(cudaMemcpyAsync(c.pos.p, positions, n3 * 8, cudaMemcpyHostToDevice, c.stream));
    CUDA_CHECK(cudaMemsetAsync(c.forcesOut.p, 0, n3 * 8, c.stream));
    c.evaluate_device(c.pos.p, box, c.forcesOut.p, nullptr);
}

int mpid_get_system_multipole_moments(mpid_context* ctx, const double* positions, const double* box,
                                      const double* masses, double* out) {
    MPID_API_BEGIN
    if (!ctx || !positions || !box || !masses || !out) throw Error(MPID_ERR_INVALID, "null argument");
    mpid::DeviceScope scope(ctx->ctx.device);
    evaluate_at(ctx->ctx, positions, box);
    ctx->ctx.system_moments(masses, out);
    return MPID_OK;
    MPID_API_END
}

int mpid_get_electrostatic_potential(mpid_context* ctx, const double* positions, const double* box,
                                     const double* grid, int ngrid, double* out) {
    MPID_API_BEGIN
    if (!ctx || !positions || !box || (ngrid > 0 && (!grid || !out))) throw Error(MPID_ERR_INVALID, "null argument");
    mpid::DeviceScope scope(ctx->ctx.device);
    evaluate_at(ctx->ctx, positions, box);
    ctx->ctx.electrostatic_potential(grid, ngrid, out);
    return MPID_OK;
    MPID_API_END
}

int mpid_get_parameter_gradients(mpid_context* ctx, const double* positions, const double* box, double* out) {
    MPID_API_BEGIN
    if (!ctx || !positions || !box || !out) throw Error(MPID_ERR_INVALID, "null argument");
    mpid::DeviceScope scope(ctx->ctx.device);
    evaluate_at(ctx->ctx, positions, box);
    ctx->ctx.parameter_gradients(out);
    return MPID_OK;
    MPID_API_END
}

int mpid_evaluate_with_gradients(mpid_context* ctx, const double* positions, const double* box, double* forces,
                                 double* energy, double* multipole_grad, double* polarization_grad) {
    MPID_API_BEGIN
    if (!ctx || !positions || !box) throw Error(MPID_ERR_INVALID, "null argument");
    Context& c = ctx->ctx;
    mpid::DeviceScope scope(c.device);
    c.stream = c.hostStream;
    const size_t n3 = 3 * (size_t) c.n;
    CUDA_CHECK(cudaMemcpyAsync(c.pos.p, positions, n3 * 8, cudaMemcpyHostToDevice, c.stream));
    if (forces)
        CUDA_CHECK(cudaMemcpyAsync(c.forcesOut.p, forces, n3 * 8, cudaMemcpyHostToDevice, c.stream));
    else
        CUDA_CHECK(cudaMemsetAsync(c.forcesOut.p, 0, n3 * 8, c.stream));
    const double e = c.evaluate_device(c.pos.p, box, c.forcesOut.p, nullptr);
    if (forces) CUDA_CHECK(cudaMemcpyAsync(forces, c.forcesOut.p, n3 * 8, cudaMemcpyDeviceToHost, c.stream));
    c.gradients(multipole_grad, polarization_grad);
    CUDA_CHECK(cudaStreamSynchronize(c.stream));
    if (energy) *energy = e;
    return MPID_OK;
    MPID_API_END
}

// The launch of the whole-evaluation graphs of many contexts: either one parent graph
// whose children are the contexts' graphs, rebuilt when a child is captured anew or the
// set of contexts changes (keyed by context ids, which are never reused, and capture
// generations), or each context's graph on one of a pool of streams.
namespace {
struct BatchGraph {
    std::vector<unsigned long long> key;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t stream = nullptr;
    std::vector<cudaStream_t> streams;  // per-context launches
    std::vector<cudaEvent_t> joins;
    int device = -1;
    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
        key.clear();
    }
};
std::mutex g_batchMutex;
BatchGraph g_batch;
mpid::FusedBatch g_fused;
}  // namespace

// The ordinary evaluation of one context of a batch at its host inputs, into its own
// buffers (used for the first call of a context and for results a batch graph could not
// stand behind).
static double batch_fallback(Context& c, const double* positions, const double* box, const double* forces, bool mg,
                             bool pg) {
    const size_t n3 = 3 * (size_t) c.n;
    CUDA_CHECK(cudaMemcpyAsync(c.pos.p, positions, n3 * 8, cudaMemcpyHostToDevice, c.stream));
    if (forces)
        CUDA_CHECK(cudaMemcpyAsync(c.forcesOut.p, forces, n3 * 8, cudaMemcpyHostToDevice, c.stream));
    else
        CUDA_CHECK(cudaMemsetAsync(c.forcesOut.p, 0, n3 * 8, c.stream));
    const double e = c.evaluate_device(c.pos.p, box, c.forcesOut.p, nullptr);
    if (mg || pg) c.gradients_device(mg, pg);
    c.batchReady = true;
    return e;
}

int mpid_evaluate_batch(mpid_context* const* ctxs, int count, const double* const* positions, const double* const* boxes,
                        double* const* forces, double* energies, double* const* multipole_grad,
                        double* const* polarization_grad, double* type_grad, int launch_mode) {
    MPID_API_BEGIN
    if (launch_mode < -1 || launch_mode > 128) throw Error(MPID_ERR_INVALID, "launch_mode must be in -1..128");
    if (count < 0 || (count > 0 && (!ctxs || !positions || !boxes || !energies)))
        throw Error(MPID_ERR_INVALID, "null argument");
    if (count == 0) return MPID_OK;
    const int device = ctxs[0] ? ctxs[0]->ctx.device : 0;
    for (int k = 0; k < count; ++k) {
        if (!ctxs[k] || !positions[k] || !boxes[k]) throw Error(MPID_ERR_INVALID, "null argument");
        if (ctxs[k]->ctx.device != device) throw Error(MPID_ERR_INVALID, "mpid_evaluate_batch: contexts on different devices");
        if (!ctxs[k]->ctx.usePme) throw Error(MPID_ERR_INVALID, "mpid_evaluate_batch supports PME contexts only");
        for (int q = 0; q < k; ++q)
            if (ctxs[q] == ctxs[k]) throw Error(MPID_ERR_INVALID, "mpid_evaluate_batch: a context appears twice");
    }
    // per-atom gradient outputs requested, and the gradients computed (also for type sums)
    auto outMg = [&](int k) { return multipole_grad && multipole_grad[k]; };
    auto outPg = [&](int k) { return polarization_grad && polarization_grad[k]; };
    auto wantMg = [&](int k) { return type_grad || outMg(k); };
    auto wantPg = [&](int k) { return type_grad || outPg(k); };
    const int nt = ctxs[0]->ctx.ntypes;
    if (type_grad) {
        for (int k = 0; k < count; ++k)
            if (ctxs[k]->ctx.ntypes <= 0 || ctxs[k]->ctx.ntypes != nt)
                throw Error(MPID_ERR_INVALID, "type_grad: every context needs the same atom types (mpid_set_atom_types)");
        std::fill(type_grad, type_grad + (size_t) 24 * nt, 0.0);
    }
    std::vector<std::vector<double>> boxSums(type_grad ? count : 0);  // per box [nt][24]
    const bool fused = launch_mode == 0;
    if (fused) {
        for (int k = 0; k < count; ++k) {
            if (outMg(k) != outMg(0) || outPg(k) != outPg(0))
                throw Error(MPID_ERR_INVALID, "fused batch: every box must request the same gradients");
            if (ctxs[k]->ctx.n > mpid::kBlockSortMax)
                throw Error(MPID_ERR_INVALID, "fused batch: boxes of at most 4096 atoms (use launch_mode > 0)");
        }
    }
    mpid::DeviceScope scope(device);
    std::lock_guard<std::mutex> lock(g_batchMutex);
    if (g_batch.device != device) {
        g_batch.reset();
        if (g_batch.stream) cudaStreamDestroy(g_batch.stream);
        for (cudaStream_t q : g_batch.streams) cudaStreamDestroy(q);
        for (cudaEvent_t ev : g_batch.joins) cudaEventDestroy(ev);
        g_batch.stream = nullptr;
        g_batch.streams.clear();
        g_batch.joins.clear();
        g_fused.release();
        g_batch.device = device;
        g_fused.device = device;
        CUDA_CHECK(cudaStreamCreateWithFlags(&g_batch.stream, cudaStreamNonBlocking));
        CUDA_CHECK(cudaStreamCreateWithFlags(&g_fused.stream, cudaStreamNonBlocking));
    }
    std::vector<char> graphed(count, 0);
    std::vector<double> eFallback(count, 0.0);
    bool changed = false;
    for (int k = 0; k < count; ++k) {
        Context& c = ctxs[k]->ctx;
        const bool mg = wantMg(k), pg = wantPg(k);
        const double* fin = forces ? forces[k] : nullptr;
        c.stream = c.hostStream;
        c.bind_streams();
        if (!c.batchReady) {
            eFallback[k] = batch_fallback(c, positions[k], boxes[k], fin, mg, pg);
            continue;
        }
        // per-box graphs: inputs on the box's stream (the fused graph copies them from its
        // pinned staging)
        if (!fused) {
            const size_t n3 = 3 * (size_t) c.n;
            CUDA_CHECK(cudaMemcpyAsync(c.pos.p, positions[k], n3 * 8, cudaMemcpyHostToDevice, c.stream));
            if (fin)
                CUDA_CHECK(cudaMemcpyAsync(c.forcesOut.p, fin, n3 * 8, cudaMemcpyHostToDevice, c.stream));
            else
                CUDA_CHECK(cudaMemsetAsync(c.forcesOut.p, 0, n3 * 8, c.stream));
        }
        c.set_box(boxes[k]);
        c.stats.graph_captures = 0;
        if (!fused) {
            changed = c.ensure_batch_graph(mg, pg) || changed;
            CUDA_CHECK(cudaStreamSynchronize(c.stream));
        }
        graphed[k] = 1;
    }
    long long launches = 0, library = 0;
    float fusedMs = 0.f;
    std::vector<int> slot(count, -1);  // a fused box's index in the staging
    if (fused) {
        // every box records the same number of CG iterations: the most any box needs
        std::vector<Context*> run;
        int K = 0;
        for (int k = 0; k < count; ++k)
            if (graphed[k]) {
                slot[k] = (int) run.size();
                run.push_back(&ctxs[k]->ctx);
                K = std::max(K, ctxs[k]->ctx.batch_iterations());
            }
        std::vector<unsigned long long> key;
        const bool mg = wantMg(0), pg = wantPg(0);
        key.push_back((outMg(0) ? 1 : 0) | (outPg(0) ? 2 : 0) | (type_grad ? 4 : 0) | ((unsigned long long) nt << 8));
        for (Context* c : run) {
            changed = c->ensure_recording(mg, pg, K) || changed;
            key.push_back(c->id);
            key.push_back(c->recGeneration);
        }
        if (!run.empty()) {
            if (changed || g_fused.key != key || !g_fused.exec) {
                mpid::fused_build(g_fused, run, outMg(0), outPg(0), type_grad != nullptr);
                g_fused.key = key;
                for (Context* c : run) ++c->stats.graph_captures;
            }
            for (int k = 0; k < count; ++k) {
                if (slot[k] < 0) continue;
                const size_t n3 = 3 * (size_t) ctxs[k]->ctx.n;
                double* in = g_fused.hostIn + g_fused.inOff[slot[k]];
                std::memcpy(in, positions[k], n3 * 8);
                if (forces && forces[k])
                    std::memcpy(in + n3, forces[k], n3 * 8);
                else
                    std::memset(in + n3, 0, n3 * 8);
            }
            CUDA_CHECK(cudaEventRecord(g_fused.evStart, g_fused.stream));
            CUDA_CHECK(cudaGraphLaunch(g_fused.exec, g_fused.stream));
            CUDA_CHECK(cudaEventRecord(g_fused.evStop, g_fused.stream));
            CUDA_CHECK(cudaStreamSynchronize(g_fused.stream));
            CUDA_CHECK(cudaEventElapsedTime(&fusedMs, g_fused.evStart, g_fused.evStop));
            for (const auto& hc : g_fused.hostCopies) std::memcpy(hc.dst, g_fused.hostOut + hc.offset, hc.bytes);
            launches = g_fused.launches;
            library = g_fused.library;
        }
    } else {
        // the parent graph of the graphed contexts
        std::vector<unsigned long long> key;
        for (int k = 0; k < count; ++k)
            if (graphed[k]) {
                key.push_back(ctxs[k]->ctx.id);
                key.push_back(ctxs[k]->ctx.full.generation);
            }
        const int streams = launch_mode;
        if (!key.empty() && streams > 0) {
            // each context's graph on one of `streams` streams, joined into the batch stream
            while ((int) g_batch.streams.size() < streams) {
                cudaStream_t q;
                cudaEvent_t ev;
                CUDA_CHECK(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
                CUDA_CHECK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
                g_batch.streams.push_back(q);
                g_batch.joins.push_back(ev);
            }
            int j = 0;
            for (int k = 0; k < count; ++k)
                if (graphed[k]) {
                    Context& c = ctxs[k]->ctx;
                    if (!c.full.exec) CUDA_CHECK(cudaGraphInstantiate(&c.full.exec, c.full.graph, 0));
                    CUDA_CHECK(cudaGraphLaunch(c.full.exec, g_batch.streams[j % streams]));
                    ++j;
                }
            for (int q = 0; q < std::min(j, streams); ++q) {
                CUDA_CHECK(cudaEventRecord(g_batch.joins[q], g_batch.streams[q]));
                CUDA_CHECK(cudaStreamWaitEvent(g_batch.stream, g_batch.joins[q], 0));
            }
            CUDA_CHECK(cudaStreamSynchronize(g_batch.stream));
        } else if (!key.empty()) {
            if (changed || g_batch.key != key || !g_batch.exec) {
                g_batch.reset();
                cudaGraph_t parent = nullptr;
                CUDA_CHECK(cudaGraphCreate(&parent, 0));
                for (int k = 0; k < count; ++k)
                    if (graphed[k]) {
                        cudaGraphNode_t node;
                        const cudaError_t rc = cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, ctxs[k]->ctx.full.graph);
                        if (rc != cudaSuccess) {
                            cudaGraphDestroy(parent);
                            CUDA_CHECK(rc);
                        }
                    }
                const cudaError_t rc = cudaGraphInstantiate(&g_batch.exec, parent, 0);
                cudaGraphDestroy(parent);
                CUDA_CHECK(rc);
                g_batch.key = key;
            }
            CUDA_CHECK(cudaGraphLaunch(g_batch.exec, g_batch.stream));
            CUDA_CHECK(cudaStreamSynchronize(g_batch.stream));
        }
    }
    // results, and the ordinary evaluation of any context whose batched results do not stand
    for (int k = 0; k < count; ++k) {
        Context& c = ctxs[k]->ctx;
        const bool mg = wantMg(k), pg = wantPg(k);
        double e = eFallback[k];
        if (graphed[k]) {
            const bool ok = fused ? c.batch_ok(launches, library) : c.batch_ok(c.full.nodes, c.full.library);
            if (ok) {
                e = c.stats.energy_parts[0] + c.stats.energy_parts[1] + c.stats.energy_parts[2];
                if (fused) {
                    // the whole fused launch's device time, and the outputs from the staging
                    c.stats.ms_total = fusedMs;
                    const size_t n = (size_t) c.n;
                    const double* out = g_fused.hostOut + g_fused.outOff[slot[k]];
                    if (forces && forces[k]) std::memcpy(forces[k], out, 3 * n * 8);
                    size_t o = 3 * n;
                    if (outMg(k)) {
                        std::memcpy(multipole_grad[k], out + o, 20 * n * 8);
                        o += 20 * n;
                    }
                    if (outPg(k)) {
                        std::memcpy(polarization_grad[k], out + o, 4 * n * 8);
                        o += 4 * n;
                    }
                    if (type_grad) boxSums[k].assign(out + o, out + o + (size_t) 24 * nt);
                    energies[k] = e;
                    continue;
                }
            } else {
                // recorded or captured anew with the new list shape or solver length
                c.full.destroy();
                c.rec.ops.clear();
                e = batch_fallback(c, positions[k], boxes[k], forces ? forces[k] : nullptr, mg, pg);
            }
        }
        energies[k] = e;
        const size_t n = (size_t) c.n;
        if (forces && forces[k])
            CUDA_CHECK(cudaMemcpyAsync(forces[k], c.forcesOut.p, 3 * n * 8, cudaMemcpyDeviceToHost, c.stream));
        if (outMg(k))
            CUDA_CHECK(cudaMemcpyAsync(multipole_grad[k], c.gradOut.p, 20 * n * 8, cudaMemcpyDeviceToHost, c.stream));
        if (outPg(k))
            CUDA_CHECK(cudaMemcpyAsync(polarization_grad[k], c.polOut.p, 4 * n * 8, cudaMemcpyDeviceToHost, c.stream));
        if (type_grad) {
            // per-type sums on the host from this box's per-atom gradients
            std::vector<double> g(20 * n), q(4 * n);
            CUDA_CHECK(cudaMemcpyAsync(g.data(), c.gradOut.p, 20 * n * 8, cudaMemcpyDeviceToHost, c.stream));
            CUDA_CHECK(cudaMemcpyAsync(q.data(), c.polOut.p, 4 * n * 8, cudaMemcpyDeviceToHost, c.stream));
            CUDA_CHECK(cudaStreamSynchronize(c.stream));
            boxSums[k].assign((size_t) 24 * nt, 0.0);
            for (size_t a = 0; a < n; ++a) {
                double* row = boxSums[k].data() + 24 * (size_t) c.atomTypesHost[a];
                for (int m = 0; m < 20; ++m) row[m] += g[20 * a + m];
                for (int m = 0; m < 4; ++m) row[20 + m] += q[4 * a + m];
            }
        }
        CUDA_CHECK(cudaStreamSynchronize(c.stream));
    }
    if (type_grad)
        for (int k = 0; k < count; ++k)
            for (size_t m = 0; m < (size_t) 24 * nt; ++m) type_grad[m] += boxSums[k][m];
    return MPID_OK;
    MPID_API_END
}

int mpid_get_dipoles(mpid_context* ctx, int which, double* out) {
    MPID_API_BEGIN
    if (!ctx || !out) throw Error(MPID_ERR_INVALID, "null argument");
    mpid::DeviceScope scope(ctx->ctx.device);
    ctx->ctx.get_dipoles(which, out);
    return MPID_OK;
    MPID_API_END
}

int mpid_get_pme_parameters(mpid_context* ctx, double* alpha, int* nx, int* ny, int* nz) {
    MPID_API_BEGIN
    if (!ctx) throw Error(MPID_ERR_INVALID, "null argument");
    if (ctx->ctx.set.nonbonded_method != MPID_PME)
        throw Error(MPID_ERR_INVALID, "getPMEParametersInContext: MPIDForce is not using PME");
    if (alpha) *alpha = ctx->ctx.set.ewald_alpha;
    if (nx) *nx = ctx->ctx.set.grid[0];
    if (ny) *ny = ctx->ctx.set.grid[1];
    if (nz) *nz = ctx->ctx.set.grid[2];
    return MPID_OK;
    MPID_API_END
}

int mpid_set_work_split(mpid_context* ctx, int max_split) {
    MPID_API_BEGIN
    if (!ctx) throw Error(MPID_ERR_INVALID, "null argument");
    if (max_split < 0 || max_split > 32 || (max_split & (max_split - 1)) != 0)
        throw Error(MPID_ERR_INVALID, "max_split must be 0 or a power of two up to 32");
    ctx->ctx.splitCap = max_split;
    return MPID_OK;
    MPID_API_END
}

int mpid_get_stats(mpid_context* ctx, mpid_stats* out) {
    MPID_API_BEGIN
    if (!ctx || !out) throw Error(MPID_ERR_INVALID, "null argument");
    *out = ctx->ctx.stats;
    out->device_allocations = (long long) mpid::g_device_allocs.load();
    return MPID_OK;
    MPID_API_END
}

const char* mpid_last_error(void) { return g_lastError.c_str(); }

}  // extern "C"
