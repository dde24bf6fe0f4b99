// Internal declarations shared by the libemfa_cuda translation units.
// Device-side vector/complex helpers are templated on the arithmetic type
// (float for the mixed-precision path, double for the plain FP64 path).
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/emfa_cuda.h"

// ---------------------------------------------------------------------------
// error plumbing: every CUDA call inside the library goes through EMFA_CUDA,
// which records the failing call on the context and returns EMFA_ERR_CUDA.
// ---------------------------------------------------------------------------
namespace emfa {

struct Ctx;
void set_error(Ctx* ctx, const std::string& msg);
void set_global_error(const std::string& msg);

#define EMFA_CUDA(ctx, call)                                                              \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            ::emfa::set_error((ctx), std::string(#call) + ": " + cudaGetErrorString(e_)); \
            return EMFA_ERR_CUDA;                                                         \
        }                                                                                 \
    } while (0)

#define EMFA_TRY(expr)                     \
    do {                                   \
        emfa_status_t s_ = (expr);         \
        if (s_ != EMFA_OK) return s_;      \
    } while (0)

// ---------------------------------------------------------------------------
// context: device, stream, HBM budget accounting, reusable workspaces
// ---------------------------------------------------------------------------
emfa_status_t ctx_alloc(Ctx* c, size_t bytes, void** p);
void ctx_free(Ctx* c, void* p, size_t bytes);

// RAII device buffer tied to a context's budget.
struct DevBuf {
    Ctx* ctx = nullptr;
    void* ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : ctx(o.ctx), ptr(o.ptr), bytes(o.bytes)
    {
        o.ptr = nullptr;
        o.bytes = 0;
    }
    ~DevBuf() { release(); }
    emfa_status_t alloc(Ctx* c, size_t b)
    {
        release();
        ctx = c;
        if (b == 0) return EMFA_OK;
        emfa_status_t s = ctx_alloc(c, b, &ptr);
        if (s == EMFA_OK) bytes = b;
        return s;
    }
    void release()
    {
        if (ptr) ctx_free(ctx, ptr, bytes);
        ptr = nullptr;
        bytes = 0;
    }
};

template <typename T> inline T* dptr(const DevBuf& b) { return reinterpret_cast<T*>(b.ptr); }
// a region of a DevBuf (not owning)
struct DevView {
    void* ptr = nullptr;
    size_t bytes = 0;
};
template <typename T> inline T* dptr(const DevView& b) { return reinterpret_cast<T*>(b.ptr); }

// Workspace slots: buffers a context keeps between calls so repeated fills,
// products and solves do not allocate.  A slot grows when a call needs more.
enum WorkspaceSlot {
    WS_GEMM_B = 0, WS_GEMM_ERR, WS_KRYLOV, WS_FILL, WS_RCS, WS_ZPLANES, WS_HGEMM,
    WS_DENSE_Z, WS_DENSE_V, WS_DENSE_X,  // emfa_dense_rcs: the job's matrix, excitation and currents
    WS_LU_WAVE,                          // tickets and flags of the LU's triangular solves
    WS_COUNT
};

// Kernels the context can time with CUDA events (emfa_ctx_set_kernel_timing).
enum KernelTimerId { KT_FILL_Z = 0, KT_GEMM, KT_RESIDUAL, KT_COUNT };

struct KernelTimer {
    std::vector<cudaEvent_t> start, stop;  // one pair per timed launch
    size_t used = 0;
    double work = 0.0;  // algorithmic FLOPs (products) or entries (fill) of the recorded launches
};

struct Ctx {
    // Handles that hold this context: the caller's (until emfa_ctx_destroy)
    // and one per live geometry or MLFMA operator.  The stream, events and the
    // struct itself go when the last one is dropped, so a child destroyed after
    // its context (finalizers in any order) still finds them.
    int refs = 1;
    int device = 0;
    size_t budget = 0;      // bytes the context may hold (0 = unlimited)
    size_t used = 0;
    size_t peak = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    std::mutex mu;
    int sm_count = 0;
    long long kernel_launches = 0;  // kernels launched through this context
    bool stream_ordered = false;  // allocations on `stream` (cudaMallocAsync), for lanes of the server
    cudaMemPool_t pool = nullptr;  // with stream_ordered: the pool to allocate from (null: the device's)
    bool time_kernels = false;
    KernelTimer timers[KT_COUNT];
    DevBuf ws[WS_COUNT];            // declared after mu: destroyed before it
    std::map<void*, size_t> user_bufs;  // emfa_device_alloc'ed buffers
    int* pinned = nullptr;          // page-locked host words for asynchronous status reads (64 ints)
};

emfa_status_t ctx_workspace(Ctx* c, int slot, size_t bytes, void** p);

// Reference counting of a context by the objects created on it (ctx.cu).
void ctx_retain(Ctx* c);
void ctx_release(Ctx* c);

// Raises the kernel's dynamic shared-memory limit on the context's device to
// at least `bytes`; the limit never goes down.  Lanes of the server launch
// the same kernels concurrently with different sizes, and a limit lowered by
// one lane between another lane's raise and its launch fails that launch.
emfa_status_t ensure_smem_raw(Ctx* c, const void* func, size_t bytes);
template <typename F>
inline emfa_status_t ensure_smem(Ctx* c, F* func, size_t bytes)
{
    return ensure_smem_raw(c, reinterpret_cast<const void*>(func), bytes);
}

// Programmatic dependent launch: a kernel launched with
// cudaLaunchAttributeProgrammaticStreamSerialization may be scheduled once
// every CTA of its predecessor has called griddep_launch (or exited), and
// waits in griddep_wait until the predecessor has finished and its writes are
// visible.  Both are no-ops for kernels launched without the attribute.
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_dependent(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                    Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Brackets one kernel launch with events on its stream when the context's
// kernel timing is on; does nothing otherwise.
class TimedLaunch {
public:
    TimedLaunch(Ctx* c, int id, cudaStream_t st, double work);
    ~TimedLaunch();

private:
    Ctx* c_;
    cudaStream_t st_;
    cudaEvent_t stop_ = nullptr;
};

// carve 256-byte aligned sub-buffers out of one workspace
struct Carver {
    char* base;
    size_t off = 0;
    template <typename T> T* take(size_t count)
    {
        off = (off + 255) & ~(size_t)255;
        T* p = reinterpret_cast<T*>(base + off);
        off += sizeof(T) * count;
        return p;
    }
    static size_t round(size_t b) { return (b + 255) & ~(size_t)255; }
};

// ---------------------------------------------------------------------------
// geometry: host copy + per-precision device pack
// ---------------------------------------------------------------------------
// Per-RWG record consumed by the fill, excitation and far-field kernels.
// Side 0 is the + triangle (RWG current leaves the free vertex vxp), side 1
// the - triangle.  All coordinates are in the kernel's arithmetic type and
// computed from that type's vertices in the reference's operation order.
template <typename T>
struct RwgPack {
    T q3[2][3][3];   // 3-point Gauss points of the two triangles
    T v[2][3];       // free vertices vxp, vxm
    T n[2][3];       // unit normals of the two triangles
    T cen[2][3];     // triangle centroids (EFIE far-pair test and EDM)
    T len;           // edge length
    int tri[2];      // triangle ids tp, tm
    int e[2];        // local index (0..2) of the free vertex in each triangle
};

template <typename T>
struct GeomDev {
    bool ready = false;
    DevBuf block;     // one allocation holding the arrays below
    DevView verts;    // V x 3
    DevView tris;     // T x 3 int
    DevView tri_q3;   // T x 3 x 3
    DevView tri_q7;   // T x 7 x 3
    DevView tri_n;    // T x 3
    DevView tri_area;  // T
    DevView rwg;      // N x RwgPack<T>
    DevView rwg_tab;  // N x 6 int, the RWG table as uploaded
};

struct Geom {
    Ctx* ctx = nullptr;
    int refs = 1;  // the caller's handle + one per MLFMA operator built on it
    int nv = 0, nt = 0, n = 0;
    std::vector<double> verts;   // host, V x 3
    std::vector<int> tris;       // host, T x 3
    std::vector<int> rwg;        // host, N x 6 (v1 v2 vxp vxm tp tm)
    DevBuf vd;                   // device copy of verts (FP64), uploaded once
    bool nbr_ready = false;      // edge neighbours of each triangle (3 int, -1 where none),
    DevBuf nbr;                  //   for the configuration's discretisation
    GeomDev<float> g32;
    GeomDev<double> g64;
    // tiled fill: the distinct triangles of each block of 16 consecutive
    // RWGs, and each RWG's position of its two triangles in its block's list
    bool tile_ready = false;
    int tile_maxt = 0;
    DevBuf tile_block;  // one allocation holding the three arrays below
    DevView tile_tris;  // int [blocks][tile_maxt]
    DevView tile_nt;    // int [blocks]
    DevView tile_loc;   // uint8 [N][2]
};

// the FP64 vertices on the device (uploaded on first use)
emfa_status_t geom_vd(Geom* g, cudaStream_t st);

emfa_status_t geom_prepare_f32(Geom* g, cudaStream_t st);
emfa_status_t geom_prepare_f64(Geom* g, cudaStream_t st);
// Reference counting of a geometry by the MLFMA operators built on it
// (geom.cu); the last release frees it and drops its hold on the context.
void geom_retain(Geom* g);
void geom_release(Geom* g);

// RWG (common edge) construction, EMComponent/CommonEdge.cpp:74-106,704-743
int build_rwg_host(const int* tris, int n_tri, std::vector<int>& rwg_out, std::string* err);

// physical constants in the arithmetic type, as EMComponent/Mathdef.h
// computes them: PI = (T)pi, Z0 = 120 PI, k = (2 PI) f / c0.
template <typename T> struct Phys {
    static T pi() { return (T)3.14159265358979323846; }
    static T z0() { return (T)120 * pi(); }
    static T c0() { return (T)299792458.0; }
    static T wavenumber(double freq) { return ((T)2 * pi()) * (T)freq / c0(); }
};

// incidence vectors k_hat, e_hat, h_hat (EMSolver/EM.cpp:33-38), 9 values
template <typename T>
void incidence_vectors(double theta_deg, double phi_deg, double pole_deg, T out[9]);

// ---------------------------------------------------------------------------
// kernel launchers (fill.cu, rcs.cu, gemm.cu, krylov.cu)
// ---------------------------------------------------------------------------
emfa_status_t launch_fill_z(Ctx* c, Geom* g, const emfa_fill_params_t* p, void* Z, size_t ldz,
                            cudaStream_t st);
emfa_status_t launch_fill_v(Ctx* c, Geom* g, const emfa_fill_params_t* p, const double* angles,
                            int n_inc, void* V, cudaStream_t st);
emfa_status_t launch_rcs(Ctx* c, Geom* g, const emfa_fill_params_t* p, const void* I, int n_rhs,
                         const double* dirs, int n_dir, int per_rhs_dirs, double* out_db,
                         cudaStream_t st);

}  // namespace emfa

struct emfa_ctx : emfa::Ctx {};
struct emfa_geom : emfa::Geom {};
