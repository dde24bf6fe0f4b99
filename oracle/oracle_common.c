/*
 * oracle_common.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * Integer parts of the oracle: the RWG (common-edge) table restated from
 * CommonEdge::buildCommonEdge / updateCommonEdge
 * (EMComponent/CommonEdge.cpp:74-106, 704-743), with the reference's own
 * O(E*T) scan so its order and orientation are the reference's by
 * construction.  Used by tests to check the product's hash-based builder.
 */
#include <stdlib.h>

typedef struct {
    int v1, v2, vxp, vxm, tp, tm;
} sce_t;

/* rwg_out: capacity cap rows of 6 ints (v1 v2 vxp vxm tp tm).
 * Returns the number of interior edges (RWGs), or -1 if cap is too small. */
int or_build_rwg(const int* tris, int nt, int* rwg_out, int cap)
{
    sce_t* tmp = (sce_t*)malloc(sizeof(sce_t) * (size_t)(3 * nt + 3));
    int ne = 0;
    for (int t = 0; t < nt; ++t) {
        int nA = tris[3 * t], nB = tris[3 * t + 1], nC = tris[3 * t + 2];
        int e1 = 1, e2 = 1, e3 = 1;
        int edge_num = ne;
        for (int i = 0; i < edge_num; ++i) {
            if (tmp[i].tm != -1) continue;
            int v1 = tmp[i].v1, v2 = tmp[i].v2;
            if (nA == v2 && nB == v1) {
                e1 = 0; tmp[i].vxm = nC; tmp[i].tm = t;
            } else if (nB == v2 && nC == v1) {
                e2 = 0; tmp[i].vxm = nA; tmp[i].tm = t;
            } else if (nC == v2 && nA == v1) {
                e3 = 0; tmp[i].vxm = nB; tmp[i].tm = t;
            }
        }
        if (e1) { sce_t s = {nA, nB, nC, -1, t, -1}; tmp[ne++] = s; }
        if (e2) { sce_t s = {nB, nC, nA, -1, t, -1}; tmp[ne++] = s; }
        if (e3) { sce_t s = {nC, nA, nB, -1, t, -1}; tmp[ne++] = s; }
    }
    int n = 0;
    for (int i = 0; i < ne; ++i) {
        if (tmp[i].tm == -1) continue; /* boundary edge: dropped */
        if (n >= cap) { free(tmp); return -1; }
        int* r = rwg_out + 6 * n;
        r[0] = tmp[i].v1; r[1] = tmp[i].v2; r[2] = tmp[i].vxp;
        r[3] = tmp[i].vxm; r[4] = tmp[i].tp; r[5] = tmp[i].tm;
        ++n;
    }
    free(tmp);
    return n;
}
