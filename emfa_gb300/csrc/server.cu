// Batched and served RCS solves (emfa_serve): many independent problems on
// one GPU.  No counterpart in the reference, which runs one problem per
// process (solver::loadSolver, EMSolver/Solver.cpp:45-95).
//
//   lanes      worker host threads, each with its own context (stream,
//              workspaces, stream-ordered device memory), so the fills,
//              products and solves of different problems overlap on the GPU
//   admitter   a request becomes visible at its arrival time; a free lane
//              takes the oldest visible request whose device-memory estimate
//              fits in what the running requests leave of the budget, else
//              the oldest one that fits; a request that has waited
//              max_wait_s holds later ones back until it fits; a request
//              larger than the whole budget runs alone once nothing else does
//   memory     lanes allocate stream-ordered from one memory pool created for
//              the run (not the device's default pool, which other users of
//              cudaMallocAsync in the process share), destroyed at its end
//   methods    dense up to dense_max unknowns: fill, then CFIE split-FP16
//              GMRES(30)-IR to 1e-6, EFIE FP32 LU with FP64 refinement to
//              1e-5 by default, then RCS; MLFMA (CFIE operator, GMRES(30) to
//              1e-3 in box order) above; each problem keeps its operators and
//              Krylov state on its lane until it finishes
#include "emfa_internal.cuh"
#include "gemm.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdint>
#include <limits>
#include <thread>
#include <vector>

namespace emfa {
namespace {

using Clock = std::chrono::steady_clock;

struct Engine {
    const emfa_request_t* reqs = nullptr;
    emfa_request_result_t* res = nullptr;
    int n = 0;
    emfa_serve_opts_t o{};
    int device = 0;
    std::vector<int> order;  // request indices by arrival time
    std::vector<double> arr; // arrival times (all 0 when not realtime)
    std::vector<size_t> est;
    std::vector<int> method;
    std::vector<char> taken;
    size_t in_use = 0;
    int running = 0;
    int unassigned = 0;
    std::mutex mu;
    std::condition_variable cv;
    Clock::time_point t0;
    cudaMemPool_t pool = nullptr;  // the lanes' stream-ordered allocations
    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
    double arrival(int i) const { return arr[i]; }
};

// Device bytes a request holds while it runs (upper estimates).
//   dense: Z complex64 + its two FP16 planes (16 N^2), for EFIE also the LU
//          factor (8 N^2), Krylov basis and vectors (~40 N R complex64),
//          packed right-hand sides, geometry
//   MLFMA: radiation + receive patterns (2 x 3 x complex64 x K_f, K_f <= 160
//          at a 0.25-wavelength finest box), near field (~110 entries a
//          row), level patterns (about 2 KB an unknown for each right-hand
//          side of an operator pass, at most 8), Krylov state
size_t estimate_bytes(const emfa_request_t& r, int dense_max, int* method)
{
    const double N = 1.5 * r.n_tri + 16;  // closed surface: 3 edges per triangle, each shared
    const double R = std::max(1, r.n_inc);
    int m = r.method == 1 || r.method == 2 ? r.method : (N <= dense_max ? 1 : 2);
    *method = m;
    double b;
    if (m == 1)
        b = (r.kind == EMFA_EFIE ? 24.0 : 16.0) * N * N + 40.0 * 8 * N * R + 16.0 * 2 * N * R + 2048.0 * N;
    else
        b = 2.0 * 3 * 8 * 160 * N + 110.0 * 8 * N + 2000.0 * N * std::min(R, 8.0) + 40.0 * 8 * N * R + 2048.0 * N;
    return (size_t)(b * 1.1) + (64u << 20);
}

// The oldest visible request that fits; else the oldest later one that fits;
// else, with nothing running, the oldest visible one.  Once the oldest
// visible request has waited max_wait_s without fitting, later ones are held
// back until it fits, so a large request cannot starve behind a stream of
// small ones that never lets the budget drain.
int choose(Engine& E, double t)
{
    const size_t budget = E.o.hbm_budget;
    int oldest = -1;
    for (int i : E.order) {
        if (E.taken[i]) continue;
        if (E.arrival(i) > t) break;
        if (E.in_use + E.est[i] <= budget) return i;
        if (oldest < 0) {
            oldest = i;
            if (t - E.arrival(i) >= E.o.max_wait_s) break;
        }
    }
    if (oldest >= 0 && E.running == 0) return oldest;
    return -1;
}

double next_arrival(Engine& E, double t)
{
    for (int i : E.order)
        if (!E.taken[i] && E.arrival(i) > t) return E.arrival(i);
    return std::numeric_limits<double>::infinity();
}

emfa_status_t run_dense(Ctx* c, Geom* g, const emfa_request_t& r, int n, emfa_request_result_t& o)
{
    cudaStream_t st = c->stream;
    // pairs beyond 3 wavelengths by ordinary quadrature (the reference zeroes them)
    emfa_fill_params_t fp{r.kind, EMFA_F32, r.freq, r.kind == EMFA_CFIE ? r.alpha : 1.0, 0.0, 0.0, 2};
    // EFIE (first kind) is ill-conditioned on these meshes: restarted GMRES
    // needs hundreds of iterations, so EFIE is factored (FP32 LU, FP64
    // refinement, GMRES(250)-IR if the refinement stalls) and solved to 1e-5
    // by default (the FP32 matrix resolves residuals to about 1e-6); CFIE
    // converges in tens of GMRES(30) iterations, to 1e-6
    const bool efie = r.kind == EMFA_EFIE;
    emfa_solver_params_t sp{efie ? EMFA_LU : EMFA_GMRES, efie ? 250 : 30,
                            r.max_iter > 0 ? r.max_iter : (efie ? 5000 : 3000), r.tol > 0 ? r.tol : (efie ? 1e-5 : 1e-6),
                            0, EMFA_MV_AUTO, 0, 0};
    DevBuf Z, V, X;
    EMFA_TRY(Z.alloc(c, 8 * (size_t)n * n));
    EMFA_TRY(V.alloc(c, 8 * (size_t)n * r.n_inc));
    EMFA_TRY(X.alloc(c, 16 * (size_t)n * r.n_inc));
    EMFA_TRY(launch_fill_z(c, g, &fp, Z.ptr, n, st));
    EMFA_TRY(launch_fill_v(c, g, &fp, r.angles, r.n_inc, V.ptr, st));
    emfa_solve_info_t info{};
    emfa_status_t s = solve_dense(c, EMFA_F32, Z.ptr, n, V.ptr, r.n_inc, X.ptr, &sp, &info, st);
    o.iterations = info.iterations;
    o.converged = info.converged;
    o.max_rel_residual = info.max_rel_residual;
    if (s != EMFA_OK && s != EMFA_ERR_NOT_CONVERGED) return s;
    if (r.rcs_out && r.rcs_dirs && r.n_dir > 0)
        EMFA_TRY(launch_rcs(c, g, &fp, X.ptr, r.n_inc, r.rcs_dirs, r.n_dir, r.per_rhs_dirs, r.rcs_out, st));
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    return s;
}

emfa_status_t run_mlfma(Ctx* c, Geom* g, const emfa_request_t& r, int n, emfa_request_result_t& o)
{
    cudaStream_t st = c->stream;
    const double alpha = r.kind == EMFA_CFIE ? r.alpha : 1.0;
    emfa_mlfma_params_t mp{r.freq, alpha, r.box_threshold > 0 ? r.box_threshold : 0.25, 0, 0.9, 0.87};
    emfa_mlfma_t* M = nullptr;
    EMFA_TRY(emfa_mlfma_create(static_cast<emfa_ctx_t*>(c), static_cast<emfa_geom_t*>(g), &mp, &M));
    struct Guard {
        emfa_mlfma_t* m;
        ~Guard() { emfa_mlfma_destroy(m); }
    } guard{M};
    DevBuf V, X, Xr;
    EMFA_TRY(V.alloc(c, 8 * (size_t)n * r.n_inc));
    EMFA_TRY(X.alloc(c, 16 * (size_t)n * r.n_inc));
    EMFA_TRY(Xr.alloc(c, 16 * (size_t)n * r.n_inc));
    EMFA_TRY(emfa_mlfma_fill_v(M, r.angles, r.n_inc, V.ptr, st));
    emfa_solver_params_t sp{EMFA_GMRES, 30, r.max_iter > 0 ? r.max_iter : 600, r.tol > 0 ? r.tol : 1e-3,
                            0, EMFA_MV_AUTO, 0, 0};
    emfa_solve_info_t info{};
    emfa_status_t s = emfa_mlfma_solve(M, V.ptr, r.n_inc, X.ptr, &sp, &info, st);
    o.iterations = info.iterations;
    o.converged = info.converged;
    o.max_rel_residual = info.max_rel_residual;
    if (s != EMFA_OK && s != EMFA_ERR_NOT_CONVERGED) return s;
    EMFA_TRY(emfa_mlfma_unpermute(M, X.ptr, r.n_inc, Xr.ptr, st));
    emfa_fill_params_t fp{EMFA_CFIE, EMFA_F32, r.freq, alpha, 0.0, 0.0, 0};
    if (r.rcs_out && r.rcs_dirs && r.n_dir > 0)
        EMFA_TRY(launch_rcs(c, g, &fp, Xr.ptr, r.n_inc, r.rcs_dirs, r.n_dir, r.per_rhs_dirs, r.rcs_out, st));
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    return s;
}

emfa_status_t run_request(Ctx* c, Engine& E, int i, emfa_request_result_t& o)
{
    const emfa_request_t& r = E.reqs[i];
    if (!r.verts || !r.tris || r.n_vert <= 0 || r.n_tri <= 0 || !r.angles || r.n_inc <= 0 || !(r.freq > 0) ||
        (r.kind != EMFA_EFIE && r.kind != EMFA_CFIE)) {
        set_error(c, "emfa_serve: bad request");
        return EMFA_ERR_INVALID;
    }
    std::vector<int> rwg;
    std::string err;
    const int n = build_rwg_host(r.tris, r.n_tri, rwg, &err);
    if (n <= 0) {
        set_error(c, "emfa_serve: no RWG unknowns (" + err + ")");
        return EMFA_ERR_MESH;
    }
    o.n_rwg = n;
    emfa_geom_t* g = nullptr;
    EMFA_TRY(emfa_geom_create(static_cast<emfa_ctx_t*>(c), r.verts, r.n_vert, r.tris, r.n_tri, rwg.data(), n, &g));
    struct Guard {
        emfa_geom_t* g;
        ~Guard() { emfa_geom_destroy(g); }
    } guard{g};
    const int dense_max = E.o.dense_max;
    const int m = r.method == 1 || r.method == 2 ? r.method : (n <= dense_max ? 1 : 2);
    o.method = m;
    return m == 1 ? run_dense(c, g, r, n, o) : run_mlfma(c, g, r, n, o);
}

void lane_main(Engine* E, int lane)
{
    cudaSetDevice(E->device);
    emfa_ctx_t* ctx = nullptr;
    const emfa_status_t cs = emfa_ctx_create(E->device, 0, &ctx);
    if (cs == EMFA_OK) {
        ctx->stream_ordered = true;
        ctx->pool = E->pool;
    }
    for (;;) {
        int pick = -1;
        {
            std::unique_lock<std::mutex> lk(E->mu);
            for (;;) {
                if (E->unassigned == 0) break;
                const double t = E->now();
                pick = choose(*E, t);
                if (pick >= 0) {
                    E->taken[pick] = 1;
                    E->in_use += E->est[pick];
                    E->running += 1;
                    E->unassigned -= 1;
                    break;
                }
                const double nx = next_arrival(*E, t);
                if (std::isinf(nx))
                    E->cv.wait_for(lk, std::chrono::milliseconds(50));
                else
                    E->cv.wait_for(lk, std::chrono::duration<double>(std::max(0.0, nx - t)));
            }
        }
        if (pick < 0) break;
        emfa_request_result_t& o = E->res[pick];
        o.lane = lane;
        o.hbm_estimate = E->est[pick];
        o.t_arrive = E->arrival(pick);
        o.t_start = E->now();
        o.status = cs != EMFA_OK ? cs : run_request(ctx, *E, pick, o);
        o.t_done = E->now();
        {
            std::lock_guard<std::mutex> lk(E->mu);
            E->in_use -= E->est[pick];
            E->running -= 1;
        }
        E->cv.notify_all();
    }
    if (ctx) emfa_ctx_destroy(ctx);
}

}  // namespace
}  // namespace emfa

using namespace emfa;

extern "C" emfa_status_t emfa_serve(int device, const emfa_request_t* reqs, int n_req, const emfa_serve_opts_t* opts,
                                    emfa_request_result_t* results)
{
    if (!reqs || n_req <= 0 || !results) {
        set_error(nullptr, "emfa_serve: bad arguments");
        return EMFA_ERR_INVALID;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        set_error(nullptr, "emfa_serve: no such CUDA device");
        return EMFA_ERR_CUDA;
    }
    Engine E;
    E.reqs = reqs;
    E.res = results;
    E.n = n_req;
    E.device = device;
    if (opts) E.o = *opts;
    if (E.o.lanes <= 0) E.o.lanes = 6;
    E.o.lanes = std::min(E.o.lanes, 64);
    if (E.o.hbm_budget == 0) E.o.hbm_budget = (size_t)150 << 30;
    if (E.o.dense_max <= 0) E.o.dense_max = 10000;
    if (!(E.o.max_wait_s > 0)) E.o.max_wait_s = 2.0;
    E.est.resize(n_req);
    E.method.resize(n_req);
    E.arr.resize(n_req);
    E.taken.assign(n_req, 0);
    E.unassigned = n_req;
    for (int i = 0; i < n_req; ++i) {
        results[i] = emfa_request_result_t{};
        results[i].status = EMFA_ERR_INVALID;
        E.est[i] = estimate_bytes(reqs[i], E.o.dense_max, &E.method[i]);
        E.arr[i] = E.o.realtime ? reqs[i].arrival_s : 0.0;
        E.order.push_back(i);
    }
    // by arrival; requests that arrive together (a whole batch) largest
    // first, so no large problem starts last and runs alone
    std::stable_sort(E.order.begin(), E.order.end(), [&](int a, int b) {
        if (E.arrival(a) != E.arrival(b)) return E.arrival(a) < E.arrival(b);
        return E.est[a] > E.est[b];
    });
    // lanes free and reallocate per problem: a pool of the run's own keeps
    // freed memory for the next problem (release threshold at its maximum);
    // it is destroyed, with what it holds, when the run ends
    cudaSetDevice(device);
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    EMFA_CUDA(nullptr, cudaMemPoolCreate(&E.pool, &props));
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(E.pool, cudaMemPoolAttrReleaseThreshold, &thr);
    E.t0 = Clock::now();
    std::vector<std::thread> th;
    for (int l = 0; l < E.o.lanes; ++l) th.emplace_back(lane_main, &E, l);
    for (auto& t : th) t.join();
    cudaDeviceSynchronize();  // the lanes' asynchronous frees have completed
    cudaMemPoolDestroy(E.pool);
    return EMFA_OK;
}

extern "C" emfa_status_t emfa_serve_simulate(const double* arrival, const double* duration, const size_t* bytes,
                                             int n, const emfa_serve_opts_t* opts, double* start_out, int* lane_out)
{
    if (!arrival || !duration || !bytes || n <= 0 || !start_out || !lane_out) return EMFA_ERR_INVALID;
    Engine E;
    E.n = n;
    if (opts) E.o = *opts;
    if (E.o.lanes <= 0) E.o.lanes = 6;
    if (E.o.hbm_budget == 0) E.o.hbm_budget = (size_t)150 << 30;
    if (!(E.o.max_wait_s > 0)) E.o.max_wait_s = 2.0;
    E.est.assign(bytes, bytes + n);
    E.arr.resize(n);
    E.taken.assign(n, 0);
    for (int i = 0; i < n; ++i) {
        E.arr[i] = E.o.realtime ? arrival[i] : 0.0;
        E.order.push_back(i);
    }
    std::stable_sort(E.order.begin(), E.order.end(), [&](int a, int b) {
        if (E.arr[a] != E.arr[b]) return E.arr[a] < E.arr[b];
        return E.est[a] > E.est[b];
    });
    std::vector<double> free_at(E.o.lanes, 0.0);
    std::vector<std::pair<double, int>> run;  // (end time, request)
    double t = 0.0;
    int assigned = 0;
    while (assigned < n) {
        const int l = (int)(std::min_element(free_at.begin(), free_at.end()) - free_at.begin());
        t = std::max(t, free_at[l]);
        for (size_t k = 0; k < run.size();) {  // finished requests give their memory back
            if (run[k].first <= t) {
                E.in_use -= E.est[run[k].second];
                E.running -= 1;
                run[k] = run.back();
                run.pop_back();
            } else {
                ++k;
            }
        }
        const int pick = choose(E, t);
        if (pick < 0) {
            double nx = next_arrival(E, t);
            for (auto& r : run) nx = std::min(nx, r.first);
            if (std::isinf(nx)) return EMFA_ERR_INVALID;  // cannot happen: something is visible or running
            t = nx;
            continue;
        }
        E.taken[pick] = 1;
        E.in_use += E.est[pick];
        E.running += 1;
        start_out[pick] = t;
        lane_out[pick] = l;
        free_at[l] = t + duration[pick];
        run.emplace_back(free_at[l], pick);
        ++assigned;
    }
    return EMFA_OK;
}
