// Geometry: RWG table construction (host), mesh upload and the per-precision
// geometry pack (Gauss points, normals, centroids, edge lengths) built on the
// device.  This translation unit is compiled with -fmad=false so the pack
// reproduces the reference's own rounding of those quantities.
#include "emfa_internal.cuh"
#include "emfa_math.cuh"

#include <cmath>
#include <unordered_map>

namespace emfa {

// CommonEdge::updateCommonEdge (EMComponent/CommonEdge.cpp:704-743) scans
// every open edge for each triangle; an edge (A,B) of a triangle pairs with
// an open edge (B,A) of an earlier one.  The same matching through a hash of
// the open directed edges, same order and orientation: RWGs are the paired
// edges in order of first appearance, + side = first triangle, free vertices
// = the opposite corners.  Boundary (never paired) edges are dropped.
int build_rwg_host(const int* tris, int n_tri, std::vector<int>& out, std::string* err)
{
    // Open half-edges by directed key (u, v), in an open-addressing table
    // whose slots head a chain of the half-edges with that key (a manifold
    // mesh has one); a triangle that brings the reverse edge (v, u) closes
    // every half-edge of the chain and frees the key.
    struct Tmp { int v1, v2, vxp, vxm, tp, tm; };
    std::vector<Tmp> tmp;
    tmp.reserve((size_t)3 * n_tri);
    std::vector<int> nxt;  // next half-edge of the same key, -1 at the end
    nxt.reserve((size_t)3 * n_tri);
    size_t cap = 16;
    while (cap < (size_t)6 * n_tri) cap <<= 1;
    const uint64_t EMPTY = ~0ull, GONE = ~0ull - 1;  // no vertex index reaches these keys
    struct Slot { uint64_t key; int head, tail; };     // one cache access per probe
    std::vector<Slot> tab(cap, Slot{EMPTY, -1, -1});
    auto key = [](int a, int b) { return ((uint64_t)(uint32_t)a << 32) | (uint32_t)b; };
    auto slot_of = [&](uint64_t k) {
        uint64_t h = k * 0x9E3779B97F4A7C15ull;
        return (size_t)(h >> 20) & (cap - 1);
    };
    auto find = [&](uint64_t k) -> long {
        for (size_t i = slot_of(k);; i = (i + 1) & (cap - 1)) {
            if (tab[i].key == k) return (long)i;
            if (tab[i].key == EMPTY) return -1;
        }
    };
    for (int t = 0; t < n_tri; ++t) {
        int a = tris[3 * t], b = tris[3 * t + 1], c = tris[3 * t + 2];
        int corner[3][3] = {{a, b, c}, {b, c, a}, {c, a, b}};
        bool fresh[3] = {true, true, true};
        for (int e = 0; e < 3; ++e) {
            const long sl = find(key(corner[e][1], corner[e][0]));
            if (sl < 0) continue;
            for (int idx = tab[sl].head; idx >= 0; idx = nxt[idx]) {
                tmp[idx].vxm = corner[e][2];
                tmp[idx].tm = t;
            }
            fresh[e] = false;
            tab[sl].key = GONE;
        }
        for (int e = 0; e < 3; ++e) {
            if (!fresh[e]) continue;
            int u = corner[e][0], v = corner[e][1];
            if (u == v) {
                if (err) *err = "degenerate triangle " + std::to_string(t);
                return -1;
            }
            const uint64_t k = key(u, v);
            const int idx = (int)tmp.size();
            tmp.push_back(Tmp{u, v, corner[e][2], -1, t, -1});
            nxt.push_back(-1);
            const long sl = find(k);
            if (sl >= 0) {  // a chain: append, keeping the order of insertion
                nxt[tab[sl].tail] = idx;
                tab[sl].tail = idx;
                continue;
            }
            size_t i = slot_of(k);
            while (tab[i].key != EMPTY && tab[i].key != GONE) i = (i + 1) & (cap - 1);
            tab[i] = Slot{k, idx, idx};
        }
    }
    out.clear();
    out.reserve(tmp.size() * 6);
    for (const Tmp& s : tmp) {
        if (s.tm == -1) continue;
        out.insert(out.end(), {s.v1, s.v2, s.vxp, s.vxm, s.tp, s.tm});
    }
    return (int)(out.size() / 6);
}

template <typename T>
void incidence_vectors(double theta_deg, double phi_deg, double pole_deg, T out[9])
{
    // EMSolver/EM.cpp:29-38.  Angles in the arithmetic type; the reference's
    // unqualified sin/cos are the C double functions, so each component is a
    // double expression rounded once to T.
    const T pi = Phys<T>::pi();
    const T d2r = pi / T(180);
    T pol = (T)pole_deg * d2r, th = (T)theta_deg * d2r, ph = (T)phi_deg * d2r;
    double st = std::sin((double)th), ct = std::cos((double)th), sp = std::sin((double)ph), cp = std::cos((double)ph);
    double so = std::sin((double)pol), co = std::cos((double)pol);
    V3<T> k = v3<T>((T)(-st * cp), (T)(-st * sp), (T)(-ct));
    V3<T> e = v3<T>((T)(-co * ct * cp - so * sp), (T)(-co * ct * sp + so * cp), (T)(co * st));
    V3<T> h = cross(k, e);
    T v[9] = {k.x, k.y, k.z, e.x, e.y, e.z, h.x, h.y, h.z};
    for (int i = 0; i < 9; ++i) out[i] = v[i];
}
template void incidence_vectors<float>(double, double, double, float*);
template void incidence_vectors<double>(double, double, double, double*);

// one thread per triangle: vertices, Gauss points, normal, area
template <typename T>
__global__ void k_pack_tris(const double* __restrict__ vd, const int* __restrict__ tris, int nt,
                            T* __restrict__ vt, T* __restrict__ q3, T* __restrict__ q7, T* __restrict__ nrm,
                            T* __restrict__ area, int nv)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < nv) {
        vt[3 * t] = (T)vd[3 * t];
        vt[3 * t + 1] = (T)vd[3 * t + 1];
        vt[3 * t + 2] = (T)vd[3 * t + 2];
    }
    if (t >= nt) return;
    V3<T> a, b, c;
    int ia = tris[3 * t], ib = tris[3 * t + 1], ic = tris[3 * t + 2];
    a = v3<T>((T)vd[3 * ia], (T)vd[3 * ia + 1], (T)vd[3 * ia + 2]);
    b = v3<T>((T)vd[3 * ib], (T)vd[3 * ib + 1], (T)vd[3 * ib + 2]);
    c = v3<T>((T)vd[3 * ic], (T)vd[3 * ic + 1], (T)vd[3 * ic + 2]);
    V3<T> p3[3], p7[7];
    gauss3(a, b, c, p3);
    gauss7(a, b, c, p7);
    for (int i = 0; i < 3; ++i) st3(q3 + 9 * t + 3 * i, p3[i]);
    for (int i = 0; i < 7; ++i) st3(q7 + 21 * t + 3 * i, p7[i]);
    st3(nrm + 3 * t, tri_normal(a, b, c));
    area[t] = tri_area(a, b, c);
}

template <typename T>
__global__ void k_pack_rwg(const double* __restrict__ vd, const int* __restrict__ tris, const int* __restrict__ rwg,
                           int n, const T* __restrict__ q3, const T* __restrict__ nrm, RwgPack<T>* __restrict__ out)
{
    int u = blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n) return;
    const int* r = rwg + 6 * u;
    RwgPack<T> pk;
    auto vtx = [&](int i) { return v3<T>((T)vd[3 * i], (T)vd[3 * i + 1], (T)vd[3 * i + 2]); };
    for (int s = 0; s < 2; ++s) {
        int t = r[4 + s];
        int fv = r[2 + s];
        pk.tri[s] = t;
        int e = 0;
        for (int j = 0; j < 3; ++j)
            if (tris[3 * t + j] == fv) e = j;
        pk.e[s] = e;
        for (int i = 0; i < 9; ++i) (&pk.q3[s][0][0])[i] = q3[9 * t + i];
        V3<T> fvv = vtx(fv);
        pk.v[s][0] = fvv.x; pk.v[s][1] = fvv.y; pk.v[s][2] = fvv.z;
        pk.n[s][0] = nrm[3 * t]; pk.n[s][1] = nrm[3 * t + 1]; pk.n[s][2] = nrm[3 * t + 2];
        V3<T> cc = centroid(vtx(tris[3 * t]), vtx(tris[3 * t + 1]), vtx(tris[3 * t + 2]));
        pk.cen[s][0] = cc.x; pk.cen[s][1] = cc.y; pk.cen[s][2] = cc.z;
    }
    pk.len = norm(vtx(r[0]) - vtx(r[1]));
    out[u] = pk;
}

emfa_status_t geom_vd(Geom* g, cudaStream_t st)
{
    if (g->vd.ptr) return EMFA_OK;
    EMFA_TRY(g->vd.alloc(g->ctx, sizeof(double) * 3 * g->nv));
    // pageable source: the copy is staged before the call returns
    EMFA_CUDA(g->ctx, cudaMemcpyAsync(g->vd.ptr, g->verts.data(), g->vd.bytes, cudaMemcpyHostToDevice, st));
    return EMFA_OK;
}

template <typename T>
static emfa_status_t geom_prepare(Geom* g, GeomDev<T>& d, cudaStream_t st)
{
    if (d.ready) return EMFA_OK;
    Ctx* c = g->ctx;
    EMFA_TRY(geom_vd(g, st));
    DevView* parts[8] = {&d.tris, &d.verts, &d.tri_q3, &d.tri_q7, &d.tri_n, &d.tri_area, &d.rwg, &d.rwg_tab};
    const size_t sizes[8] = {sizeof(int) * 3 * (size_t)g->nt, sizeof(T) * 3 * (size_t)g->nv,
                             sizeof(T) * 9 * (size_t)g->nt,   sizeof(T) * 21 * (size_t)g->nt,
                             sizeof(T) * 3 * (size_t)g->nt,   sizeof(T) * (size_t)g->nt,
                             sizeof(RwgPack<T>) * (size_t)g->n, sizeof(int) * 6 * (size_t)g->n};
    size_t total = 0;
    for (size_t b : sizes) total += (b + 255) & ~(size_t)255;
    EMFA_TRY(d.block.alloc(c, total));
    size_t off = 0;
    for (int i = 0; i < 8; ++i) {
        parts[i]->ptr = (char*)d.block.ptr + off;
        parts[i]->bytes = sizes[i];
        off += (sizes[i] + 255) & ~(size_t)255;
    }
    EMFA_CUDA(c, cudaMemcpyAsync(d.tris.ptr, g->tris.data(), d.tris.bytes, cudaMemcpyHostToDevice, st));
    EMFA_CUDA(c, cudaMemcpyAsync(d.rwg_tab.ptr, g->rwg.data(), d.rwg_tab.bytes, cudaMemcpyHostToDevice, st));
    int m = g->nt > g->nv ? g->nt : g->nv;
    k_pack_tris<T><<<(m + 127) / 128, 128, 0, st>>>(dptr<double>(g->vd), dptr<int>(d.tris), g->nt, dptr<T>(d.verts),
                                                    dptr<T>(d.tri_q3), dptr<T>(d.tri_q7), dptr<T>(d.tri_n),
                                                    dptr<T>(d.tri_area), g->nv);
    k_pack_rwg<T><<<(g->n + 127) / 128, 128, 0, st>>>(dptr<double>(g->vd), dptr<int>(d.tris), dptr<int>(d.rwg_tab),
                                                      g->n, dptr<T>(d.tri_q3), dptr<T>(d.tri_n),
                                                      dptr<RwgPack<T>>(d.rwg));
    c->kernel_launches += 2;
    EMFA_CUDA(c, cudaGetLastError());
    // later users may run on other streams: the arrays are complete on return
    EMFA_CUDA(c, cudaStreamSynchronize(st));
    d.ready = true;
    return EMFA_OK;
}

emfa_status_t geom_prepare_f32(Geom* g, cudaStream_t st) { return geom_prepare<float>(g, g->g32, st); }
emfa_status_t geom_prepare_f64(Geom* g, cudaStream_t st) { return geom_prepare<double>(g, g->g64, st); }

void geom_retain(Geom* g)
{
    std::lock_guard<std::mutex> lk(g->ctx->mu);
    g->refs += 1;
}

// The geometry's device arrays are freed through its context, which it
// holds until then; the context may already be closed by its caller.
void geom_release(Geom* g)
{
    Ctx* c = g->ctx;
    {
        std::lock_guard<std::mutex> lk(c->mu);
        if (--g->refs > 0) return;
    }
    cudaSetDevice(c->device);
    delete static_cast<emfa_geom_t*>(g);
    ctx_release(c);
}

}  // namespace emfa

using namespace emfa;

extern "C" {

emfa_status_t emfa_build_rwg(const int* tris_host, int n_tri, int* rwg_host, int capacity, int* n_rwg)
{
    if (!tris_host || n_tri <= 0 || !n_rwg) {
        set_global_error("emfa_build_rwg: bad arguments");
        return EMFA_ERR_INVALID;
    }
    std::vector<int> out;
    std::string err;
    int n = build_rwg_host(tris_host, n_tri, out, &err);
    if (n < 0) {
        set_global_error("emfa_build_rwg: " + err);
        return EMFA_ERR_MESH;
    }
    *n_rwg = n;
    if (n > capacity || !rwg_host) {
        set_global_error("emfa_build_rwg: capacity too small");
        return EMFA_ERR_INVALID;
    }
    std::copy(out.begin(), out.end(), rwg_host);
    return EMFA_OK;
}

emfa_status_t emfa_geom_create(emfa_ctx_t* ctx, const double* verts_host, int n_vert, const int* tris_host,
                               int n_tri, const int* rwg_host, int n_rwg, emfa_geom_t** out)
{
    if (!ctx || !verts_host || !tris_host || !rwg_host || !out || n_vert <= 0 || n_tri <= 0 || n_rwg <= 0) {
        set_error(ctx, "emfa_geom_create: bad arguments");
        return EMFA_ERR_INVALID;
    }
    for (int i = 0; i < 3 * n_tri; ++i)
        if (tris_host[i] < 0 || tris_host[i] >= n_vert) {
            set_error(ctx, "emfa_geom_create: triangle vertex index out of range");
            return EMFA_ERR_MESH;
        }
    for (int u = 0; u < n_rwg; ++u) {
        const int* r = rwg_host + 6 * u;
        for (int j = 0; j < 4; ++j)
            if (r[j] < 0 || r[j] >= n_vert) {
                set_error(ctx, "emfa_geom_create: RWG vertex index out of range (open edge?)");
                return EMFA_ERR_MESH;
            }
        for (int j = 4; j < 6; ++j)
            if (r[j] < 0 || r[j] >= n_tri) {
                set_error(ctx, "emfa_geom_create: RWG triangle index out of range");
                return EMFA_ERR_MESH;
            }
    }
    emfa_geom_t* g = new emfa_geom_t();
    g->ctx = ctx;
    ctx_retain(ctx);
    g->nv = n_vert;
    g->nt = n_tri;
    g->n = n_rwg;
    g->verts.assign(verts_host, verts_host + 3 * (size_t)n_vert);
    g->tris.assign(tris_host, tris_host + 3 * (size_t)n_tri);
    g->rwg.assign(rwg_host, rwg_host + 6 * (size_t)n_rwg);
    *out = g;
    return EMFA_OK;
}

emfa_status_t emfa_geom_destroy(emfa_geom_t* geom)
{
    if (!geom) return EMFA_ERR_INVALID;
    geom_release(geom);
    return EMFA_OK;
}

emfa_status_t emfa_geom_size(const emfa_geom_t* geom, int* n_vert, int* n_tri, int* n_rwg)
{
    if (!geom) return EMFA_ERR_INVALID;
    if (n_vert) *n_vert = geom->nv;
    if (n_tri) *n_tri = geom->nt;
    if (n_rwg) *n_rwg = geom->n;
    return EMFA_OK;
}

}  // extern "C"
