// Test-only harness around the reference's own solver classes (EFIE, CFIE,
// MLFMA of xiangwei0909/EMFA).  It is compiled together with the reference
// sources by oracle/build_ref.sh and dumps what those classes compute, in
// binary, so tests can pin the oracle restatement and the GPU path to the
// reference itself.  Nothing in the product links or runs this file.
//
//   emfa_ref_<f32|f64> rwg   <config> <outdir>
//   emfa_ref_<f32|f64> efie  <config> <outdir> <gmres_tol>
//   emfa_ref_<f32|f64> cfie  <config> <outdir> <bicgstab_tol>
//   emfa_ref_<f32|f64> mlfma <config> <outdir> <seed>
//   emfa_ref_<f32|f64> time  <config> <efie|cfie> <rows> <solve:0|1>
//   emfa_ref_<f32|f64> stages <config> <rows> <gemv_reps>
//   emfa_ref_<f32|f64> big   <config> <outdir> <efie|cfie> <incfile> [solve:0|1]
//   emfa_ref_<f32|f64> job   <config>
//   emfa_ref_<f32|f64> rcs_of <config> <outdir> <efie|cfie> <ifile> <dirfile> <mono|bi|config>
//
// The harness calls the same member functions EFIE::solve (EFIE.cpp:54-99),
// CFIE::solve (CFIE.cpp:53-88) and MLFMA::solve (MLFMA.cpp:67-106) call, in
// the same order, and reads the members they fill.
#include "Custom.h"
#include <thread>
#include <mutex>
#include <condition_variable>
#include <functional>
#include <queue>
#include <atomic>
#include <chrono>
#include <list>
#include <unordered_map>
#include <random>
#include <array>
#include <string>
#include <cstdio>
#include <cstring>
#include <experimental/filesystem>
#include "Mathdef.h"
#include "Quadrature.h"
#include "VectorC3.h"
#define private public
#define protected public
#include "ConfigLoader.h"
#include "Mesh.h"
#include "CommonEdge.h"
#include "Result.h"
#include "EFIE.h"
#include "CFIE.h"
#include "MLFMA.h"
#include "iml.h"
#undef private
#undef protected

using namespace component;
using namespace mom;

static std::string g_out;

template <typename T>
static void dump(const char* name, const T* data, size_t n)
{
    std::string p = g_out + "/" + name;
    FILE* f = std::fopen(p.c_str(), "wb");
    if (!f) { std::perror(p.c_str()); std::exit(2); }
    std::fwrite(data, sizeof(T), n, f);
    std::fclose(f);
}

template <typename S>
static void dump_geometry(S& s)
{
    auto& mesh = *s.mesh_ptr_;
    auto& ce = *s.ce_ptr_;
    int nv = mesh.getNodeNum(), nt = mesh.getTriangleNum(), n = ce.getCommonEdgeNum();
    std::vector<value_t> verts(3 * nv), normals(3 * nt), len(n);
    std::vector<int> tris(3 * nt), rwg(6 * n);
    for (int i = 0; i < nv; ++i) {
        auto& v = mesh.getVertex(i);
        verts[3 * i] = v.x; verts[3 * i + 1] = v.y; verts[3 * i + 2] = v.z;
    }
    for (int t = 0; t < nt; ++t) {
        auto& tr = mesh.getTriangleRef(t);
        tr.getVertex(tris[3 * t], tris[3 * t + 1], tris[3 * t + 2]);
        auto& nm = tr.getNormal();
        normals[3 * t] = nm.x; normals[3 * t + 1] = nm.y; normals[3 * t + 2] = nm.z;
    }
    for (int u = 0; u < n; ++u) {
        int v1, v2, vp, vm, fp, fm;
        value_t l;
        ce.getCommonEdge(u, v1, v2);
        ce.getCommonEdge(u, vp, vm, fp, fm, l);
        int* r = &rwg[6 * u];
        r[0] = v1; r[1] = v2; r[2] = vp; r[3] = vm; r[4] = fp; r[5] = fm;
        len[u] = l;
    }
    dump("verts.bin", verts.data(), verts.size());
    dump("tris.bin", tris.data(), tris.size());
    dump("normals.bin", normals.data(), normals.size());
    dump("rwg.bin", rwg.data(), rwg.size());
    dump("rwg_len.bin", len.data(), len.size());
    int meta[3] = {nv, nt, n};
    dump("meta.bin", meta, 3);
}

// Directions of Result::getBistaticRCS (Result.h:59-98): one phi cut over
// theta_from..theta_to, then the theta = 90 ring phi = 0..359.
static std::vector<VectorR3> rcs_directions(const Scattering& sca)
{
    std::vector<VectorR3> dirs;
    value_t phi = sca.phi_from * DegreesToRadians;
    value_t cosp = cos(phi), sinp = sin(phi);
    for (value_t td = sca.theta_from; td <= sca.theta_to; td += sca.theta_delta) {
        value_t th = td * DegreesToRadians;
        dirs.emplace_back(sin(th) * cosp, sin(th) * sinp, cos(th));
    }
    for (value_t pd = 0; pd < 360; pd += 1) {
        value_t p = pd * DegreesToRadians;
        dirs.emplace_back(cos(p), sin(p), 0);
    }
    return dirs;
}

template <typename S>
static void dump_rcs(S& s)
{
    auto dirs = rcs_directions(s.scattering_);
    std::vector<value_t> out(dirs.size()), kd(3 * dirs.size());
    for (size_t i = 0; i < dirs.size(); ++i) {
        out[i] = s.getBiRCS(dirs[i]);
        kd[3 * i] = dirs[i].x; kd[3 * i + 1] = dirs[i].y; kd[3 * i + 2] = dirs[i].z;
    }
    dump("rcs.bin", out.data(), out.size());
    dump("rcs_dirs.bin", kd.data(), kd.size());
}

static void dump_inc(const EM& s, value_t k)
{
    value_t v[10] = {s.inc_k_.x, s.inc_k_.y, s.inc_k_.z, s.inc_e_.x, s.inc_e_.y, s.inc_e_.z,
                     s.inc_h_.x, s.inc_h_.y, s.inc_h_.z, k};
    dump("inc.bin", v, 10);
}

static int run_efie(ConfigLoader& loader, double tol)
{
    EFIE s;
    s.init(&loader);
    dump_geometry(s);
    dump_inc(s, s.k_);
    int n = s.unknowns_;
    s.Z.zeros(n, n);
    s.Z_eigen.setZero(n, n);
    s.fillZ();
    std::vector<Complex> zb((size_t)n * n), ze((size_t)n * n);
    for (int f = 0; f < n; ++f)
        for (int c = 0; c < n; ++c) {
            zb[(size_t)f * n + c] = s.Z(f, c);
            ze[(size_t)f * n + c] = s.Z_eigen(f, c);
        }
    dump("Z_arma.bin", zb.data(), zb.size());
    dump("Z.bin", ze.data(), ze.size());
    s.I.zeros(n); s.V.zeros(n);
    s.I_eigen.setZero(n); s.V_eigen.setZero(n);
    s.fillV();
    dump("V.bin", s.V_eigen.data(), n);
    if (tol > 0) {
        iml::GMRES(s.Z_eigen, s.V_eigen, s.I_eigen, (value_t)tol, 30, 5);
        dump("I.bin", s.I_eigen.data(), n);
        dump_rcs(s);
        Result result;
        result.getBistaticRCS(&s, &EFIE::getBiRCS);
    }
    return 0;
}

static int run_cfie(ConfigLoader& loader, double tol)
{
    CFIE s;
    s.init(&loader);
    dump_geometry(s);
    dump_inc(s, s.k_);
    int n = s.unknowns_;
    s.fillZ();
    std::vector<Complex> zb((size_t)n * n);
    for (int f = 0; f < n; ++f)
        for (int c = 0; c < n; ++c) zb[(size_t)f * n + c] = s.Z(f, c);
    dump("Z.bin", zb.data(), zb.size());
    s.fillV();
    dump("V.bin", s.V.memptr(), n);
    if (tol > 0) {
        int iters = 0;
        iml::BICGSTAB(s.Z, s.V, s.I, (value_t)tol, 500, iters);
        dump("I.bin", s.I.memptr(), n);
        int it[1] = {iters};
        dump("iters.bin", it, 1);
        dump_rcs(s);
        Result result;
        result.getBistaticRCS(&s, &CFIE::getBiRCS);
    }
    return 0;
}

static int run_mlfma(ConfigLoader& loader, unsigned seed)
{
    MLFMA s;
    s.init(&loader);
    dump_geometry(s);
    dump_inc(s, s.k_);
    int n = s.unknowns_;
    int L = s.level_;
    // box order of the unknowns and the finest-level tree
    std::vector<int> perm;
    for (auto& b : s.level_box_.back())
        for (int u : b.unknown) perm.push_back(u);
    dump("perm.bin", perm.data(), perm.size());
    std::vector<int> lvl_boxes;
    for (int l = 0; l <= L; ++l) lvl_boxes.push_back((int)s.level_box_[l].size());
    dump("level_boxes.bin", lvl_boxes.data(), lvl_boxes.size());
    std::vector<value_t> blen(s.box_len_.begin(), s.box_len_.end());
    dump("box_len.bin", blen.data(), blen.size());
    // per level box table: offset, count, parent index, center, #near, #far
    for (int l = 2; l <= L; ++l) {
        std::vector<double> tab;
        for (auto& b : s.level_box_[l]) {
            tab.push_back((double)b.offset);
            tab.push_back((double)b.unknown.size());
            tab.push_back(l > 2 ? (double)b.parent->index : -1.0);
            tab.push_back(b.center.x); tab.push_back(b.center.y); tab.push_back(b.center.z);
            tab.push_back((double)b.near.size()); tab.push_back((double)b.far.size());
        }
        char nm[64];
        std::snprintf(nm, sizeof nm, "boxes_l%d.bin", l);
        dump(nm, tab.data(), tab.size());
    }
    s.levelRootsAndWeights();
    s.calculateInterpolationMtr();
    s.calculateLevelK();
    std::vector<int> poles;
    for (auto& t : s.glxt_) poles.push_back((int)t.n_elem);
    dump("poles.bin", poles.data(), poles.size());
    s.calculateLevelTrans();
    s.calculateRadAndRecv();
    s.calculateNearZ();
    s.fillVbyBox();
    dump("V.bin", s.V_.memptr(), n);
    {   // near matrix as (row, col, value) triplets in box order
        std::vector<int> rc;
        std::vector<Complex> val;
        for (auto it = s.nearZ_.begin(); it != s.nearZ_.end(); ++it) {
            rc.push_back((int)it.row());
            rc.push_back((int)it.col());
            val.push_back(*it);
        }
        dump("near_rc.bin", rc.data(), rc.size());
        dump("near_val.bin", val.data(), val.size());
    }
    s.allocateForSolve();
    s.calculateCoeff();
    std::mt19937 gen(seed);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    Qcx_vec x(n);
    // seed 0: a closed form that numpy reproduces bit for bit (integers, then
    // one correctly rounded division), so large fixtures need not store x
    for (int i = 0; i < n; ++i)
        x(i) = seed ? Complex((value_t)U(gen), (value_t)U(gen))
                    : Complex((value_t)(((long long)i * 7919) % 2001 - 1000) / (value_t)1000,
                              (value_t)(((long long)i * 104729) % 2003 - 1001) / (value_t)1001);
    dump("mv_x.bin", x.memptr(), n);
    Qcx_vec y = s.matrixVectorMultiply(x);
    dump("mv_y.bin", y.memptr(), n);
    Qcx_vec yn = s.nearZ_ * x;
    dump("mv_near.bin", yn.memptr(), n);
    int iters = s.iterativeSolve();
    int it[1] = {iters};
    dump("iters.bin", it, 1);
    dump("I.bin", s.I_.memptr(), n);
    dump_rcs(s);
    s.clear();  // joins the ThreadPool, as solver::invoke_solver does
    return 0;
}

// Incidences for the multi-incidence modes: a text file of "theta phi pole"
// lines (degrees).  Each one is applied through the reference's own
// EM::init (EM.cpp:25-41) on the loader's dictionary, so the incidence
// vectors are the ones a config with those values gives.
static std::vector<std::array<std::string, 3>> read_incidences(const char* path)
{
    std::vector<std::array<std::string, 3>> out;
    FILE* f = std::fopen(path, "r");
    if (!f) { std::perror(path); std::exit(2); }
    char a[64], b[64], c[64];
    while (std::fscanf(f, "%63s %63s %63s", a, b, c) == 3) out.push_back({a, b, c});
    std::fclose(f);
    return out;
}

static void set_incidence(ConfigLoader& loader, EM& s, const std::array<std::string, 3>& inc)
{
    loader.dict_.at("theta:").value = inc[0];
    loader.dict_.at("phi:").value = inc[1];
    loader.dict_.at("pole:").value = inc[2];
    s.EM::init(&loader);
}

// Solver-specific access for the multi-incidence modes: EFIE solves
// Z_eigen/V_eigen/I_eigen (EFIE.cpp:79), CFIE its Armadillo Z/V/I (CFIE.cpp:76).
static void fill_z_rows(EFIE& e, int n, std::vector<Complex>& zb)
{
    e.Z.zeros(n, n);
    e.Z_eigen.setZero(n, n);
    e.fillZ();
    for (int f = 0; f < n; ++f)
        for (int c = 0; c < n; ++c) zb[(size_t)f * n + c] = e.Z_eigen(f, c);
}

static void fill_z_rows(CFIE& s, int n, std::vector<Complex>& zb)
{
    s.fillZ();
    for (int f = 0; f < n; ++f)
        for (int c = 0; c < n; ++c) zb[(size_t)f * n + c] = s.Z(f, c);
}

static const Complex* fill_v_once(EFIE& e, int n)
{
    e.V.zeros(n);
    e.V_eigen.setZero(n);
    e.fillV();
    return e.V_eigen.data();
}

static const Complex* fill_v_once(CFIE& s, int)
{
    s.fillV();
    return s.V.memptr();
}

static void set_current(EFIE& e, int n, const Complex* c)
{
    e.I_eigen.resize(n);
    for (int u = 0; u < n; ++u) e.I_eigen(u) = c[u];
}

static void set_current(CFIE& s, int n, const Complex* c)
{
    s.I.set_size(n);
    for (int u = 0; u < n; ++u) s.I(u) = c[u];
}

// Full-size dense dump: one fill, then the excitation of every incidence in
// <incfile>.  Writes Z.bin (row-major, the matrix the reference solves),
// V.bin (incidence-major), inc.bin (k, e, h, wavenumber per incidence).
static int stock_solve(EFIE&, int) { return -1; }

// CFIE::solve's own solve (CFIE.cpp:76): BiCGStab to 0.01, at most 500 steps
static int stock_solve(CFIE& s, int)
{
    int iters = 0;
    iml::BICGSTAB(s.Z, s.V, s.I, 0.01f, 500, iters);
    return iters;
}

template <typename S>
static int run_big(ConfigLoader& loader, const char* incfile, bool solve)
{
    S s;
    s.init(&loader);
    dump_geometry(s);
    int n = s.unknowns_;
    auto incs = read_incidences(incfile);
    std::vector<Complex> zb((size_t)n * n), vall;
    std::vector<value_t> incv;
    fill_z_rows(s, n, zb);
    dump("Z.bin", zb.data(), zb.size());
    std::vector<Complex>().swap(zb);
    std::vector<int> iters;
    for (auto& inc : incs) {
        set_incidence(loader, s, inc);
        const Complex* v = fill_v_once(s, n);
        vall.insert(vall.end(), v, v + n);
        if (solve) iters.push_back(stock_solve(s, n));
        value_t iv[10] = {s.inc_k_.x, s.inc_k_.y, s.inc_k_.z, s.inc_e_.x, s.inc_e_.y, s.inc_e_.z,
                          s.inc_h_.x, s.inc_h_.y, s.inc_h_.z, s.k_};
        incv.insert(incv.end(), iv, iv + 10);
    }
    dump("V.bin", vall.data(), vall.size());
    dump("inc.bin", incv.data(), incv.size());
    if (solve) dump("iters.bin", iters.data(), iters.size());
    return 0;
}

// One stock CFIE job of the reference as one process runs it, timed per
// stage with the reference's own functions in CFIE::solve / CFIE::output
// order (CFIE.cpp:53-88): init (mesh + RWG), fillZ, fillV, BiCGStab to 0.01,
// then the RCS in the monostatic direction -k_inc through getBiRCS.  Prints
// one JSON record.
static int run_job(ConfigLoader& loader)
{
    using clk = std::chrono::steady_clock;
    auto sec = [](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
    auto t0 = clk::now();
    CFIE s;
    s.init(&loader);
    const double t_init = sec(t0);
    t0 = clk::now();
    s.fillZ();
    const double t_fill = sec(t0);
    t0 = clk::now();
    s.fillV();
    const double t_fillv = sec(t0);
    t0 = clk::now();
    int iters = 0;
    const bool ok = iml::BICGSTAB(s.Z, s.V, s.I, 0.01f, 500, iters);
    const double t_solve = sec(t0);
    t0 = clk::now();
    const value_t rcs = s.getBiRCS(VectorR3(-s.inc_k_.x, -s.inc_k_.y, -s.inc_k_.z));
    const double t_rcs = sec(t0);
    std::printf("{\"n\": %d, \"init_s\": %.6f, \"fill_s\": %.6f, \"fillv_s\": %.6f, \"solve_s\": %.6f, "
                "\"rcs_s\": %.6f, \"iters\": %d, \"converged\": %d, \"rcs_db\": %.6f}\n",
                s.unknowns_, t_init, t_fill, t_fillv, t_solve, t_rcs, iters, ok ? 1 : 0, (double)rcs);
    return 0;
}

// RCS of given currents through the reference's getBiRCS (EFIE.cpp:788-832,
// CFIE.cpp:643-685): <ifile> holds n_cur currents of the solver's order
// (binary Complex), <dirfile> n_dir directions (x y z per line).  "mono":
// current i at direction i (n_cur == n_dir); "bi": every current at every
// direction; "config": every current at the config's bistatic directions
// (dirfile unused).
template <typename S>
static int run_rcs_of(ConfigLoader& loader, const char* ifile, const char* dirfile, const std::string& pairing)
{
    S s;
    s.init(&loader);
    int n = s.unknowns_;
    std::vector<Complex> cur;
    {
        FILE* f = std::fopen(ifile, "rb");
        if (!f) { std::perror(ifile); std::exit(2); }
        Complex c;
        while (std::fread(&c, sizeof c, 1, f) == 1) cur.push_back(c);
        std::fclose(f);
    }
    std::vector<VectorR3> dirs;
    if (pairing == "config") {  // the config's bistatic directions (Result.h:59-98)
        dirs = rcs_directions(s.scattering_);
        std::vector<value_t> kd;
        for (auto& d : dirs) { kd.push_back(d.x); kd.push_back(d.y); kd.push_back(d.z); }
        dump("rcs_dirs.bin", kd.data(), kd.size());
    } else {
        FILE* f = std::fopen(dirfile, "r");
        if (!f) { std::perror(dirfile); std::exit(2); }
        double x, y, z;
        while (std::fscanf(f, "%lf %lf %lf", &x, &y, &z) == 3)
            dirs.emplace_back((value_t)x, (value_t)y, (value_t)z);
        std::fclose(f);
    }
    size_t n_cur = cur.size() / n;
    if (pairing == "mono" && n_cur != dirs.size()) {
        std::fprintf(stderr, "rcs_of: %zu currents, %zu directions\n", n_cur, dirs.size());
        return 1;
    }
    std::vector<value_t> out;
    for (size_t i = 0; i < n_cur; ++i) {
        set_current(s, n, &cur[i * n]);
        if (pairing == "mono") {
            out.push_back(s.getBiRCS(dirs[i]));
        } else {
            for (auto& d : dirs) out.push_back(s.getBiRCS(d));
        }
    }
    dump("rcs.bin", out.data(), out.size());
    return 0;
}

// Wall time of the reference fill on its leading rows x rows block: the
// outer and inner loops of EFIE::fillZ / CFIE::fillZ both run to unknowns_,
// so lowering unknowns_ bounds the sample; every entry costs the same work
// as in the full fill (all kernels, singular terms where they fall).  With
// solve=1 the full-size fill, RHS and Krylov solve run as the reference runs
// them (BiCGStab 1e-2 for CFIE, GMRES 1e-3 for EFIE).
static int run_time(ConfigLoader& loader, const std::string& kind, int rows, int solve)
{
    using clk = std::chrono::steady_clock;
    double fill_s = 0, solve_s = 0, full_fill_s = 0;
    int n = 0;
    if (kind == "cfie") {
        CFIE s;
        s.init(&loader);
        n = s.unknowns_;
        s.unknowns_ = rows < n ? rows : n;
        auto t0 = clk::now();
        s.fillZ();
        fill_s = std::chrono::duration<double>(clk::now() - t0).count();
        s.unknowns_ = n;
        if (solve) {
            auto t1 = clk::now();
            s.fillZ();
            full_fill_s = std::chrono::duration<double>(clk::now() - t1).count();
            s.fillV();
            auto t2 = clk::now();
            int iters = 0;
            iml::BICGSTAB(s.Z, s.V, s.I, 0.01f, 500, iters);
            solve_s = std::chrono::duration<double>(clk::now() - t2).count();
        }
    } else {
        EFIE s;
        s.init(&loader);
        n = s.unknowns_;
        s.unknowns_ = rows < n ? rows : n;
        s.Z.zeros(s.unknowns_, s.unknowns_);
        s.Z_eigen.setZero(s.unknowns_, s.unknowns_);
        auto t0 = clk::now();
        s.fillZ();
        fill_s = std::chrono::duration<double>(clk::now() - t0).count();
        s.unknowns_ = n;
    }
    std::printf("{\"n\": %d, \"rows\": %d, \"fill_s\": %.6f, \"full_fill_s\": %.6f, \"solve_s\": %.6f}\n",
                n, rows < n ? rows : n, fill_s, full_fill_s, solve_s);
    return 0;
}

// Per-stage wall times of the reference's CFIE path on a bounded sample:
// mesh + RWG init, the leading rows x rows block of the fill, fillV, one
// Armadillo complex GEMV of the full order (the product iml::BICGSTAB runs
// twice per iteration, EMIterative/iml.cpp:22,29) and getBiRCS for one
// direction.  The caller scales these to the full job.
static int run_stages(ConfigLoader& loader, int rows, int reps)
{
    using clk = std::chrono::steady_clock;
    auto sec = [](clk::time_point a) { return std::chrono::duration<double>(clk::now() - a).count(); };
    auto t0 = clk::now();
    CFIE s;
    s.init(&loader);
    double t_init = sec(t0);
    int n = s.unknowns_;
    s.unknowns_ = rows < n ? rows : n;
    t0 = clk::now();
    s.fillZ();
    double t_block = sec(t0);
    s.unknowns_ = n;
    t0 = clk::now();
    s.fillV();
    double t_fillv = sec(t0);
    Qcx_mat Z(n, n);
    std::mt19937 gen(3);
    std::uniform_real_distribution<float> U(-1.0f, 1.0f);
    for (size_t i = 0; i < Z.n_elem; ++i) Z(i) = Complex(U(gen), U(gen));
    Qcx_vec x(n), y(n);
    for (int i = 0; i < n; ++i) x(i) = Complex(U(gen), U(gen));
    y = Z * x;  // warm
    t0 = clk::now();
    for (int r = 0; r < reps; ++r) y = Z * x;
    double t_gemv = sec(t0) / reps;
    s.I = x;
    t0 = clk::now();
    volatile value_t v = s.getBiRCS(VectorR3(1, 0, 0));
    (void)v;
    double t_rcs = sec(t0);
    std::printf("{\"n\": %d, \"rows\": %d, \"init_s\": %.6f, \"block_fill_s\": %.6f, \"fillv_s\": %.6f, "
                "\"gemv_s\": %.6f, \"rcs_dir_s\": %.6f}\n",
                n, rows < n ? rows : n, t_init, t_block, t_fillv, t_gemv, t_rcs);
    s.clear();
    return 0;
}

int main(int argc, char** argv)
{
    if (argc < 3 || (argc < 4 && std::string(argv[1]) != "job")) {
        std::fprintf(stderr, "usage: %s rwg|efie|cfie|mlfma|time|stages|big|rcs_of|job <config> ...\n", argv[0]);
        return 1;
    }
    std::string mode = argv[1];
    ConfigLoader loader;
    try {
        loader.load(argv[2]);
        if (mode == "time")
            return run_time(loader, argv[3], argc > 4 ? std::atoi(argv[4]) : 64, argc > 5 ? std::atoi(argv[5]) : 0);
        if (mode == "job") return run_job(loader);
        if (mode == "stages")
            return run_stages(loader, std::atoi(argv[3]), argc > 4 ? std::atoi(argv[4]) : 3);
        g_out = argv[3];
        std::experimental::filesystem::create_directories(g_out);
        if (mode == "rwg") {
            EFIE s;
            s.init(&loader);
            dump_geometry(s);
            return 0;
        }
        if (mode == "efie") return run_efie(loader, argc > 4 ? std::atof(argv[4]) : 1e-3);
        if (mode == "cfie") return run_cfie(loader, argc > 4 ? std::atof(argv[4]) : 1e-2);
        if (mode == "mlfma") return run_mlfma(loader, argc > 4 ? (unsigned)std::atoi(argv[4]) : 1u);
        if (mode == "big" && argc > 5) {
            std::string kind = argv[4];
            const bool solve = argc > 6 && std::atoi(argv[6]) != 0;
            return kind == "efie" ? run_big<EFIE>(loader, argv[5], solve) : run_big<CFIE>(loader, argv[5], solve);
        }
        if (mode == "rcs_of" && argc > 7) {
            std::string kind = argv[4];
            return kind == "efie" ? run_rcs_of<EFIE>(loader, argv[5], argv[6], argv[7])
                                  : run_rcs_of<CFIE>(loader, argv[5], argv[6], argv[7]);
        }
    } catch (const std::exception& e) {
        std::fprintf(stderr, "reference error: %s\n", e.what());
        return 3;
    }
    std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 1;
}
