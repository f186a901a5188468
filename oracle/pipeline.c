/* CPU oracle: restatement of the reference's V0 extraction path in plain C.
 * TEST INFRASTRUCTURE ONLY -- used by tests/, smoke() and bench.py's CPU
 * baseline as the checker; never linked into the product.
 *
 * Arithmetic is written in the reference's evaluation order (compile with
 * -ffp-contract=off) so that integer outputs are bit-exact and FP outputs
 * match the reference's to the last bit where the reference's own order is
 * known.  Reference citations are to src/ of purdue-onchip/gds2Para. */
#define _POSIX_C_SOURCE 200809L
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <time.h>
#include "oracle.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
/* fdtd.hpp:45-47 */
#define MU (4 * M_PI * 1.e-7)
#define CSPED (299792458.)
#define EPSILON0 (1. / (CSPED * CSPED * MU))

typedef struct g2po_amg_handle g2po_amg_handle;
g2po_amg_handle *g2po_amg_create(const g2po_csr *A, const g2po_solver_opts *o);
int g2po_amg_solve(g2po_amg_handle *H, const double *b, double *x, const g2po_solver_opts *o,
                   g2po_solve_stats *st);
void g2po_amg_destroy(g2po_amg_handle *H);

typedef struct {
    int64_t nx, ny, nz, Nx, Ny, Nz;
    int64_t Ns, Nv, L, N_edge, N_node_s, N_node;
} dims_t;

static dims_t dims(const g2po_mesh *m) {
    /* mesh.cpp:393-402 */
    dims_t d;
    d.nx = m->nx; d.ny = m->ny; d.nz = m->nz;
    d.Nx = m->nx - 1; d.Ny = m->ny - 1; d.Nz = m->nz - 1;
    d.Ns = d.Ny * (d.Nx + 1) + d.Nx * (d.Ny + 1);
    d.Nv = (d.Nx + 1) * (d.Ny + 1);
    d.L = d.Ns + d.Nv;
    d.N_edge = d.Ns * (d.Nz + 1) + d.Nv * d.Nz;
    d.N_node_s = d.Nv;
    d.N_node = (d.Nz + 1) * d.N_node_s;
    return d;
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* ------------------------------------------------------- index maps (a3,a4) */
int64_t g2po_index_maps(const g2po_mesh *m, int64_t *map_edge, uint8_t *pec_edge, uint8_t *pec_node) {
    dims_t d = dims(m);
    memset(pec_edge, 0, (size_t)d.N_edge);
    memset(pec_node, 0, (size_t)d.N_node);
    /* findBoundNodeEdge (fdtd.hpp:1444-1505) on every node of each return
       conductor (mesh.cpp:943-953): inz==0 -> lbdn/lbde, inz==nz-1 -> ubdn/ubde,
       edges kept only where markEdge != 0. */
    for (int64_t n = 0; n < d.N_node; n++) {
        int64_t c = m->mark_node[n];
        if (c == 0 || !m->cdt_return[c - 1]) continue;
        int64_t iz = n / d.N_node_s, ix = (n % d.N_node_s) / (d.Ny + 1), iy = (n % d.N_node_s) % (d.Ny + 1);
        if (iz != 0 && iz != d.nz - 1) continue;
        pec_node[n] = 1;
        int64_t e;
        if (ix != 0) { e = iz * d.L + d.Ny * (d.Nx + 1) + (ix - 1) * (d.Ny + 1) + iy; if (m->mark_edge[e]) pec_edge[e] = 1; }
        if (ix != d.nx - 1) { e = iz * d.L + d.Ny * (d.Nx + 1) + ix * (d.Ny + 1) + iy; if (m->mark_edge[e]) pec_edge[e] = 1; }
        if (iy != 0) { e = iz * d.L + ix * d.Ny + iy - 1; if (m->mark_edge[e]) pec_edge[e] = 1; }
        if (iy != d.ny - 1) { e = iz * d.L + ix * d.Ny + iy; if (m->mark_edge[e]) pec_edge[e] = 1; }
    }
    /* LOWER_BOUNDARY_PEC (fdtd.hpp:63, mesh.cpp:963-972): the whole z=0 plane */
    for (int64_t e = 0; e < d.Ns; e++) pec_edge[e] = 1;
    for (int64_t n = 0; n < d.N_node_s; n++) pec_node[n] = 1;
    /* setMapEdge (fdtd.hpp:1508-1529) */
    int64_t count = 0;
    for (int64_t e = 0; e < d.N_edge; e++) {
        int lower = e < d.Ns && pec_edge[e];
        int upper = e >= d.N_edge - d.Ns && pec_edge[e];
        if (lower || upper) { map_edge[e] = -1; count++; }
        else map_edge[e] = e - count;
    }
    return count;
}

/* ------------------------------------------------------------ stiffness (a7-a9) */
/* Face-by-edge matrices Se and Sh in the reference's face order
 * (generateStiff.cpp:33-245 for Se, :250-484 for Sh), as CSR over faces. */
typedef struct { int64_t nf; int64_t *ptr; int64_t *edge; double *se, *sh; } faces_t;

static void faces_build(const g2po_mesh *m, faces_t *F) {
    dims_t d = dims(m);
    const double *xn = m->xn, *yn = m->yn, *zn = m->zn;
    int64_t Nx = d.Nx, Ny = d.Ny, Nz = d.Nz, L = d.L, XO = Ny * (Nx + 1), ZO = d.Ns;
    int64_t nf = Nx * Ny * (3 * Nz + 1) + Nz * Ny + Nz * Nx;
    F->nf = nf;
    F->ptr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nf + 1));
    F->edge = (int64_t *)malloc(sizeof(int64_t) * (size_t)(4 * nf));
    F->se = (double *)malloc(sizeof(double) * (size_t)(4 * nf));
    F->sh = (double *)malloc(sizeof(double) * (size_t)(4 * nf));
    double *dxa = (double *)malloc(sizeof(double) * (size_t)(Nx + 1));
    double *dya = (double *)malloc(sizeof(double) * (size_t)(Ny + 1));
    double *dza = (double *)malloc(sizeof(double) * (size_t)(Nz + 1));
    /* generateStiff.cpp:250-267 */
    dxa[0] = xn[1] - xn[0]; dya[0] = yn[1] - yn[0]; dza[0] = zn[1] - zn[0];
    dxa[Nx] = xn[Nx] - xn[Nx - 1]; dya[Ny] = yn[Ny] - yn[Ny - 1]; dza[Nz] = zn[Nz] - zn[Nz - 1];
    for (int64_t i = 1; i < Nx; i++) dxa[i] = (xn[i + 1] - xn[i - 1]) / 2;
    for (int64_t i = 1; i < Ny; i++) dya[i] = (yn[i + 1] - yn[i - 1]) / 2;
    for (int64_t i = 1; i < Nz; i++) dza[i] = (zn[i + 1] - zn[i - 1]) / 2;
#define YE(z, x, y) ((z) * L + (x) * Ny + (y))
#define XE(z, x, y) ((z) * L + XO + (x) * (Ny + 1) + (y))
#define ZE(z, x, y) ((z) * L + ZO + (x) * (Ny + 1) + (y))
    int64_t k = 0, f = 0;
#define PUT(e, a, b) do { F->edge[k] = (e); F->se[k] = (a); F->sh[k] = (b); k++; } while (0)
#define END_FACE() do { F->ptr[f] = k - 4; f++; } while (0)
    for (int64_t cz = 0; cz < Nz; cz++) {
        int top = cz == Nz - 1;
        for (int64_t cx = 0; cx < Nx; cx++) {
            for (int64_t cy = 0; cy < Ny; cy++) {
                double dx = xn[cx + 1] - xn[cx], dy = yn[cy + 1] - yn[cy], dz = zn[cz + 1] - zn[cz];
                /* xy face at plane cz */
                PUT(YE(cz, cx, cy), -1 / dx, -dza[cz] / (dxa[cx] * dza[cz]));
                PUT(YE(cz, cx + 1, cy), 1 / dx, dza[cz] / (dxa[cx + 1] * dza[cz]));
                PUT(XE(cz, cx, cy), 1 / dy, dza[cz] / (dza[cz] * dya[cy]));
                PUT(XE(cz, cx, cy + 1), -1 / dy, -dza[cz] / (dza[cz] * dya[cy + 1]));
                END_FACE();
                /* yz face at x = cx */
                PUT(YE(cz, cx, cy), 1 / dz, dxa[cx] / (dxa[cx] * dza[cz]));
                PUT(ZE(cz, cx, cy), -1 / dy, -dxa[cx] / (dxa[cx] * dya[cy]));
                PUT(ZE(cz, cx, cy + 1), 1 / dy, dxa[cx] / (dxa[cx] * dya[cy + 1]));
                PUT(YE(cz + 1, cx, cy), -1 / dz, -dxa[cx] / (dxa[cx] * dza[cz + 1]));
                END_FACE();
                /* xz face at y = cy */
                PUT(XE(cz, cx, cy), -1 / dz, -dya[cy] / (dza[cz] * dya[cy]));
                PUT(ZE(cz, cx, cy), 1 / dx, dya[cy] / (dxa[cx] * dya[cy]));
                PUT(ZE(cz, cx + 1, cy), -1 / dx, -dya[cy] / (dya[cy] * dxa[cx + 1]));
                PUT(XE(cz + 1, cx, cy), 1 / dz, dya[cy] / (dya[cy] * dza[cz + 1]));
                END_FACE();
                if (top) {
                    /* xy face at plane Nz; its Sh keeps dza[Nz-1] (generateStiff.cpp:409-427) */
                    PUT(YE(cz + 1, cx, cy), -1 / dx, -dza[cz] / (dza[cz] * dxa[cx]));
                    PUT(YE(cz + 1, cx + 1, cy), 1 / dx, dza[cz] / (dza[cz] * dxa[cx + 1]));
                    PUT(XE(cz + 1, cx, cy), 1 / dy, dza[cz] / (dza[cz] * dya[cy]));
                    PUT(XE(cz + 1, cx, cy + 1), -1 / dy, -dza[cz] / (dza[cz] * dya[cy + 1]));
                    END_FACE();
                }
            }
        }
    }
    /* rightmost yz plane x = Nx (generateStiff.cpp:193-218, :432-455) */
    for (int64_t cz = 0; cz < Nz; cz++)
        for (int64_t cy = 0; cy < Ny; cy++) {
            double dy = yn[cy + 1] - yn[cy], dz = zn[cz + 1] - zn[cz];
            PUT(YE(cz, Nx, cy), 1 / dz, dxa[Nx] / (dxa[Nx] * dza[cz]));
            PUT(ZE(cz, Nx, cy), -1 / dy, -dxa[Nx] / (dxa[Nx] * dya[cy]));
            PUT(ZE(cz, Nx, cy + 1), 1 / dy, dxa[Nx] / (dxa[Nx] * dya[cy + 1]));
            PUT(YE(cz + 1, Nx, cy), -1 / dz, -dxa[Nx] / (dxa[Nx] * dza[cz + 1]));
            END_FACE();
        }
    /* farthest xz plane y = Ny (generateStiff.cpp:221-245, :458-484) */
    for (int64_t cz = 0; cz < Nz; cz++)
        for (int64_t cx = 0; cx < Nx; cx++) {
            double dx = xn[cx + 1] - xn[cx], dz = zn[cz + 1] - zn[cz];
            PUT(XE(cz, cx, Ny), -1 / dz, -dya[Ny] / (dya[Ny] * dza[cz]));
            PUT(ZE(cz, cx, Ny), 1 / dx, dya[Ny] / (dya[Ny] * dxa[cx]));
            PUT(ZE(cz, cx + 1, Ny), -1 / dx, -dya[Ny] / (dya[Ny] * dxa[cx + 1]));
            PUT(XE(cz + 1, cx, Ny), 1 / dz, dya[Ny] / (dya[Ny] * dza[cz + 1]));
            END_FACE();
        }
    F->ptr[f] = k;
#undef PUT
#undef END_FACE
#undef YE
#undef XE
#undef ZE
    free(dxa); free(dya); free(dza);
}

static void faces_free(faces_t *F) { free(F->ptr); free(F->edge); free(F->se); free(F->sh); }

static int cmp_pair(const void *a, const void *b) {
    const int64_t x = ((const int64_t *)a)[0], y = ((const int64_t *)b)[0];
    return (x > y) - (x < y);
}

int g2po_stiffness(const g2po_mesh *m, const int64_t *map_edge, const uint8_t *pec_edge, g2po_csr *S) {
    dims_t d = dims(m);
    faces_t F;
    faces_build(m, &F);
    /* faces containing each edge, increasing face id (the transpose of the
       face-major Sh, generateStiff.cpp:507-536 -> mklMatrixMulti_nt :897-926) */
    int64_t *eptr = (int64_t *)calloc((size_t)(d.N_edge + 1), sizeof(int64_t));
    for (int64_t k = 0; k < F.ptr[F.nf]; k++) eptr[F.edge[k] + 1]++;
    for (int64_t e = 0; e < d.N_edge; e++) eptr[e + 1] += eptr[e];
    int64_t *eface = (int64_t *)malloc(sizeof(int64_t) * (size_t)eptr[d.N_edge]);
    double *esh = (double *)malloc(sizeof(double) * (size_t)eptr[d.N_edge]);
    int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)d.N_edge);
    memcpy(fill, eptr, sizeof(int64_t) * (size_t)d.N_edge);
    for (int64_t f = 0; f < F.nf; f++)
        for (int64_t k = F.ptr[f]; k < F.ptr[f + 1]; k++) {
            int64_t p = fill[F.edge[k]]++;
            eface[p] = f; esh[p] = F.sh[k];
        }
    free(fill);
    int64_t nrow = 0;
    for (int64_t e = 0; e < d.N_edge; e++) if (map_edge[e] >= 0) nrow++;
    S->n = nrow; S->m = nrow;
    S->ptr = (int64_t *)calloc((size_t)(nrow + 1), sizeof(int64_t));
    int64_t cap = nrow * 13 + 16;
    S->col = (int64_t *)malloc(sizeof(int64_t) * (size_t)cap);
    S->val = (double *)malloc(sizeof(double) * (size_t)cap);
    int64_t cols[64];
    double acc[64];
    int64_t pair[128];
    int64_t nnz = 0, r = 0;
    for (int64_t e = 0; e < d.N_edge; e++) {
        if (pec_edge[e]) continue;                   /* generateStiff.cpp:946 */
        int nc = 0;
        for (int64_t p = eptr[e]; p < eptr[e + 1]; p++) {
            int64_t f = eface[p];
            double a = esh[p];
            for (int64_t k = F.ptr[f]; k < F.ptr[f + 1]; k++) {
                int64_t j = F.edge[k];
                int t;
                for (t = 0; t < nc; t++) if (cols[t] == j) break;
                if (t == nc) { cols[nc] = j; acc[nc] = 0.0; nc++; }
                acc[t] += a * F.se[k];
            }
        }
        for (int t = 0; t < nc; t++) { pair[2 * t] = cols[t]; pair[2 * t + 1] = t; }
        qsort(pair, (size_t)nc, 2 * sizeof(int64_t), cmp_pair);     /* :953-954 */
        for (int t = 0; t < nc; t++) {
            int64_t j = pair[2 * t];
            if (pec_edge[j]) continue;                               /* :956-959 */
            S->col[nnz] = map_edge[j];
            S->val[nnz] = acc[pair[2 * t + 1]] / MU;                 /* :962 */
            nnz++;
        }
        S->ptr[++r] = nnz;
    }
    free(eptr); free(eface); free(esh);
    faces_free(&F);
    return 0;
}

/* ------------------------------------------------------------- V0 bases (a10,a12) */
/* avg_length (fdtd.hpp:4074-4104) */
static void avg_length(const g2po_mesh *m, int64_t iz, int64_t iy, int64_t ix, double *lx, double *ly, double *lz) {
    const double *xn = m->xn, *yn = m->yn, *zn = m->zn;
    if (iz == 0) *lz = zn[1] - zn[0];
    else if (iz == m->nz - 1) *lz = zn[iz] - zn[iz - 1];
    else *lz = (zn[iz + 1] - zn[iz - 1]) / 2;
    if (iy == 0) *ly = yn[1] - yn[0];
    else if (iy == m->ny - 1) *ly = yn[iy] - yn[iy - 1];
    else *ly = (yn[iy + 1] - yn[iy - 1]) / 2;
    if (ix == 0) *lx = xn[1] - xn[0];
    else if (ix == m->nx - 1) *lx = xn[ix] - xn[ix - 1];
    else *lx = (xn[ix + 1] - xn[ix - 1]) / 2;
}

typedef struct { int64_t cap; g2po_v0 *v; } v0buf;

static void v0_push(v0buf *B, int64_t row, int64_t col, double val, double aval) {
    g2po_v0 *v = B->v;
    if (v->nnz == B->cap) {
        B->cap = B->cap ? B->cap * 2 : 1024;
        v->row = (int64_t *)realloc(v->row, sizeof(int64_t) * (size_t)B->cap);
        v->col = (int64_t *)realloc(v->col, sizeof(int64_t) * (size_t)B->cap);
        v->val = (double *)realloc(v->val, sizeof(double) * (size_t)B->cap);
        v->aval = (double *)realloc(v->aval, sizeof(double) * (size_t)B->cap);
    }
    v->row[v->nnz] = row; v->col[v->nnz] = col; v->val[v->nnz] = val; v->aval[v->nnz] = aval;
    v->nnz++;
}

void g2po_v0_free(g2po_v0 *v) {
    free(v->row); free(v->col); free(v->val); free(v->aval); free(v->map);
    memset(v, 0, sizeof(*v));
}

/* The six incident edges of a node in the reference's order (lower z, upper z,
 * left x, right x, front y, back y) with the gradient value +-1/h and the
 * a-value +-1/l_avg used by V0d1 and V0c (fdtd.hpp:2524-2667, 3300-3475). */
static void node_column(const g2po_mesh *m, const dims_t *d, int64_t nd, int64_t col, v0buf *B) {
    const double *xn = m->xn, *yn = m->yn, *zn = m->zn;
    int64_t iz = nd / d->N_node_s, ix = (nd % d->N_node_s) / (d->Ny + 1), iy = (nd % d->N_node_s) % (d->Ny + 1);
    double lx, ly, lz;
    avg_length(m, iz, iy, ix, &lx, &ly, &lz);
    if (iz != 0) v0_push(B, (iz - 1) * d->L + d->Ns + ix * (d->Ny + 1) + iy, col, -1 / (zn[iz] - zn[iz - 1]), -1 / lz);
    if (iz != d->nz - 1) v0_push(B, iz * d->L + d->Ns + ix * (d->Ny + 1) + iy, col, 1 / (zn[iz + 1] - zn[iz]), 1 / lz);
    if (ix != 0) v0_push(B, iz * d->L + d->Ny * (d->Nx + 1) + (ix - 1) * (d->Ny + 1) + iy, col, -1 / (xn[ix] - xn[ix - 1]), -1 / lx);
    if (ix != d->nx - 1) v0_push(B, iz * d->L + d->Ny * (d->Nx + 1) + ix * (d->Ny + 1) + iy, col, 1 / (xn[ix + 1] - xn[ix]), 1 / lx);
    if (iy != 0) v0_push(B, iz * d->L + ix * d->Ny + iy - 1, col, -1 / (yn[iy] - yn[iy - 1]), -1 / ly);
    if (iy != d->ny - 1) v0_push(B, iz * d->L + ix * d->Ny + iy, col, 1 / (yn[iy + 1] - yn[iy]), 1 / ly);
}

int g2po_v0d(const g2po_mesh *m, const uint8_t *pec_node, g2po_v0 *v) {
    dims_t d = dims(m);
    const double *xn = m->xn, *yn = m->yn, *zn = m->zn;
    memset(v, 0, sizeof(*v));
    v->map = (int64_t *)calloc((size_t)d.N_node, sizeof(int64_t));
    v0buf B = {0, v};
    /* V0d1: with block sizes 0 (matrixCon.cpp:35-40) every dielectric node
       that is not a PEC-plane node forms its own column, in node order
       (fdtd.hpp:1866-2422, filled :2524-2667). */
    int64_t col = 0;
    for (int64_t nd = 0; nd < d.N_node; nd++) {
        int64_t iz = nd / d.N_node_s;
        int bnd = (iz == 0 || iz == d.nz - 1) && pec_node[nd];
        if (bnd || m->mark_node[nd] != 0) continue;
        v->map[nd] = col + 1;
        node_column(m, &d, nd, col, &B);
        col++;
    }
    /* V0d2 (fdtd.hpp:2424-2505 count, 2669-2759 fill): one column per
       non-reference conductor with entries on its dielectric boundary edges.
       The counting pass numbers map[] by conductors that have entries; the
       fill pass does not reset `mark` between conductors (fdtd.hpp:2673). */
    int64_t ncdt = m->num_cdt;
    int64_t *cptr = (int64_t *)calloc((size_t)(ncdt + 1), sizeof(int64_t));
    for (int64_t nd = 0; nd < d.N_node; nd++) if (m->mark_node[nd]) cptr[m->mark_node[nd]]++;
    for (int64_t c = 0; c < ncdt; c++) cptr[c + 1] += cptr[c];
    int64_t *cnodes = (int64_t *)malloc(sizeof(int64_t) * (size_t)(cptr[ncdt] + 1));
    int64_t *cfill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ncdt + 1));
    memcpy(cfill, cptr, sizeof(int64_t) * (size_t)(ncdt + 1));
    for (int64_t nd = 0; nd < d.N_node; nd++) if (m->mark_node[nd]) cnodes[cfill[m->mark_node[nd] - 1]++] = nd;
    free(cfill);
    double LX = (xn[d.nx - 1] - xn[0]) / (d.nx - 1);
    double LY = (yn[d.ny - 1] - yn[0]) / (d.ny - 1);
    double LZ = (zn[d.nz - 1] - zn[0]) / (d.nz - 1);
    int mark = 0;
    int64_t count = col;
    /* counting pass: map numbering */
    for (int64_t c = 0; c < ncdt; c++) {
        if (m->mark_port[c] == -1) continue;
        mark = 0;
        for (int64_t p = cptr[c]; p < cptr[c + 1]; p++) {
            int64_t nd = cnodes[p];
            v->map[nd] = count + 1;
            int64_t iz = nd / d.N_node_s, ix = (nd % d.N_node_s) / (d.Ny + 1), iy = (nd % d.N_node_s) % (d.Ny + 1);
            int64_t me = m->mark_node[nd], e;
            if (iz != 0) { e = (iz - 1) * d.L + d.Ns + ix * (d.Ny + 1) + iy; if (!m->mark_edge[e] && m->mark_node[nd - d.N_node_s] != me) mark = 1; }
            if (iz != d.nz - 1) { e = iz * d.L + d.Ns + ix * (d.Ny + 1) + iy; if (!m->mark_edge[e] && m->mark_node[nd + d.N_node_s] != me) mark = 1; }
            if (ix != 0) { e = iz * d.L + d.Ny * (d.Nx + 1) + (ix - 1) * (d.Ny + 1) + iy; if (!m->mark_edge[e] && m->mark_node[nd - (d.Ny + 1)] != me) mark = 1; }
            if (ix != d.nx - 1) { e = iz * d.L + d.Ny * (d.Nx + 1) + ix * (d.Ny + 1) + iy; if (!m->mark_edge[e] && m->mark_node[nd + (d.Ny + 1)] != me) mark = 1; }
            if (iy != 0) { e = iz * d.L + ix * d.Ny + iy - 1; if (!m->mark_edge[e] && m->mark_node[nd - 1] != me) mark = 1; }
            if (iy != d.ny - 1) { e = iz * d.L + ix * d.Ny + iy; if (!m->mark_edge[e] && m->mark_node[nd + 1] != me) mark = 1; }
        }
        if (mark == 1) count++;
    }
    /* fill pass */
    for (int64_t c = 0; c < ncdt; c++) {
        if (m->mark_port[c] == -1) continue;
        for (int64_t p = cptr[c]; p < cptr[c + 1]; p++) {
            int64_t nd = cnodes[p];
            int64_t iz = nd / d.N_node_s, ix = (nd % d.N_node_s) / (d.Ny + 1), iy = (nd % d.N_node_s) % (d.Ny + 1);
            int64_t me = m->mark_node[nd], e;
            double lx, ly, lz;
            avg_length(m, iz, iy, ix, &lx, &ly, &lz);
            if (iz != 0) { e = (iz - 1) * d.L + d.Ns + ix * (d.Ny + 1) + iy;
                if (!m->mark_edge[e] && m->mark_node[nd - d.N_node_s] != me) { v0_push(&B, e, col, -1 / (zn[iz] - zn[iz - 1]), -lx * ly / (LX * LY * LZ)); mark = 1; } }
            if (iz != d.nz - 1) { e = iz * d.L + d.Ns + ix * (d.Ny + 1) + iy;
                if (!m->mark_edge[e] && m->mark_node[nd + d.N_node_s] != me) { v0_push(&B, e, col, 1 / (zn[iz + 1] - zn[iz]), lx * ly / (LX * LY * LZ)); mark = 1; } }
            if (ix != 0) { e = iz * d.L + d.Ny * (d.Nx + 1) + (ix - 1) * (d.Ny + 1) + iy;
                if (!m->mark_edge[e] && m->mark_node[nd - (d.Ny + 1)] != me) { v0_push(&B, e, col, -1 / (xn[ix] - xn[ix - 1]), -ly * lz / (LX * LY * LZ)); mark = 1; } }
            if (ix != d.nx - 1) { e = iz * d.L + d.Ny * (d.Nx + 1) + ix * (d.Ny + 1) + iy;
                if (!m->mark_edge[e] && m->mark_node[nd + (d.Ny + 1)] != me) { v0_push(&B, e, col, 1 / (xn[ix + 1] - xn[ix]), ly * lz / (LX * LY * LZ)); mark = 1; } }
            if (iy != 0) { e = iz * d.L + ix * d.Ny + iy - 1;
                if (!m->mark_edge[e] && m->mark_node[nd - 1] != me) { v0_push(&B, e, col, -1 / (yn[iy] - yn[iy - 1]), -lx * lz / (LX * LY * LZ)); mark = 1; } }
            if (iy != d.ny - 1) { e = iz * d.L + ix * d.Ny + iy;
                if (!m->mark_edge[e] && m->mark_node[nd + 1] != me) { v0_push(&B, e, col, 1 / (yn[iy + 1] - yn[iy]), lx * lz / (LX * LY * LZ)); mark = 1; } }
        }
        if (mark == 1) col++;
    }
    v->ncol = col;
    free(cptr); free(cnodes);
    return 0;
}

int g2po_v0c(const g2po_mesh *m, const uint8_t *pec_node, g2po_v0 *v) {
    dims_t d = dims(m);
    memset(v, 0, sizeof(*v));
    v->map = (int64_t *)calloc((size_t)d.N_node, sizeof(int64_t));
    v0buf B = {0, v};
    int64_t ncdt = m->num_cdt;
    int64_t *cptr = (int64_t *)calloc((size_t)(ncdt + 1), sizeof(int64_t));
    for (int64_t nd = 0; nd < d.N_node; nd++) if (m->mark_node[nd]) cptr[m->mark_node[nd]]++;
    for (int64_t c = 0; c < ncdt; c++) cptr[c + 1] += cptr[c];
    int64_t *cnodes = (int64_t *)malloc(sizeof(int64_t) * (size_t)(cptr[ncdt] + 1));
    int64_t *cfill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ncdt + 1));
    memcpy(cfill, cptr, sizeof(int64_t) * (size_t)(ncdt + 1));
    for (int64_t nd = 0; nd < d.N_node; nd++) if (m->mark_node[nd]) cnodes[cfill[m->mark_node[nd] - 1]++] = nd;
    free(cfill);
    /* merge_v0c with block sizes 0 (fdtd.hpp:2900-3207): one column per
       conductor node, dropping the last node of every non-reference
       conductor and the PEC-plane nodes of reference/passive conductors. */
    int64_t col = 0;
    for (int64_t c = 0; c < ncdt; c++) {
        int64_t nn = cptr[c + 1] - cptr[c];
        int mp = m->mark_port[c];
        int64_t n = mp <= -1 ? nn : nn - 1;
        for (int64_t j = 0; j < n; j++) {
            int64_t nd = cnodes[cptr[c] + j];
            if (mp <= 0 && pec_node[nd]) continue;
            v->map[nd] = col + 1;
            node_column(m, &d, nd, col, &B);
            col++;
        }
    }
    v->ncol = col;
    free(cptr); free(cnodes);
    return 0;
}

/* -------------------------------------------------------- Ad, Ac (a11,a13) */
typedef struct { int64_t col; double val; } kv_t;

static int cmp_kv(const void *a, const void *b) {
    int64_t x = ((const kv_t *)a)->col, y = ((const kv_t *)b)->col;
    return (x > y) - (x < y);
}

/* Shared body of generateAd (fdtd.hpp:2778-2862) and generateAc
 * (fdtd.hpp:3481-3574): each V0 entry contributes to its column's row of
 * A through the other endpoint's map; unmapped endpoints add |.| to the
 * diagonal.  `coef` is stackEpsn*EPSILON0 (Ad) or stackSign (Ac). */
static int assemble_laplacian(const g2po_mesh *m, const g2po_v0 *v, int is_ac, g2po_csr *A) {
    dims_t d = dims(m);
    int64_t ncol = v->ncol;
    A->n = ncol; A->m = ncol;
    A->ptr = (int64_t *)calloc((size_t)(ncol + 1), sizeof(int64_t));
    int64_t cap = v->nnz + ncol + 16;
    A->col = (int64_t *)malloc(sizeof(int64_t) * (size_t)cap);
    A->val = (double *)malloc(sizeof(double) * (size_t)cap);
    kv_t *row = NULL;
    int64_t rowcap = 0, nnz = 0;
    /* pos[c]: slot of column c in the current row (the reference keeps an
       unordered_map per row, fdtd.hpp:2779); reset after each row */
    int64_t *pos = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ncol + 1));
    for (int64_t c = 0; c <= ncol; c++) pos[c] = -1;
    int64_t k = 0;
    for (int64_t c = 0; c < ncol; c++) {
        int64_t nr = 0;
        /* entries of column c are contiguous in the V0 COO */
        for (; k < v->nnz && v->col[k] == c; k++) {
            int64_t e = v->row[k];
            if (is_ac && m->mark_edge[e] == 0) continue;
            int64_t inz = e / d.L, r = e % d.L, n1, n2;
            double h;
            if (r >= d.Ns) {
                int64_t inx = (r - d.Ns) / (d.Ny + 1), iny = (r - d.Ns) % (d.Ny + 1);
                n1 = inz * d.N_node_s + (d.Ny + 1) * inx + iny; n2 = n1 + d.N_node_s;
                h = m->zn[inz + 1] - m->zn[inz];
            } else if (r >= d.Ny * (d.Nx + 1)) {
                int64_t inx = (r - d.Ny * (d.Nx + 1)) / (d.Ny + 1), iny = (r - d.Ny * (d.Nx + 1)) % (d.Ny + 1);
                n1 = inz * d.N_node_s + inx * (d.Ny + 1) + iny; n2 = n1 + (d.Ny + 1);
                h = m->xn[inx + 1] - m->xn[inx];
            } else {
                int64_t inx = r / d.Ny, iny = r % d.Ny;
                n1 = inz * d.N_node_s + inx * (d.Ny + 1) + iny; n2 = n1 + 1;
                h = m->yn[iny + 1] - m->yn[iny];
            }
            double a = v->aval[k];
            double off = 0.0, dg;
            int64_t other = -1;
            if (v->map[n1] != c + 1 && v->map[n1] != 0) {
                other = v->map[n1] - 1;
                if (is_ac) { off = a * 1 / h * m->stack_sign[inz]; dg = a * (-1) / h * m->stack_sign[inz]; }
                else { off = a * 1 / h * m->stack_epsn[inz] * EPSILON0; dg = a * (-1) / h * m->stack_epsn[inz] * EPSILON0; }
            } else if (v->map[n2] != c + 1 && v->map[n2] != 0) {
                other = v->map[n2] - 1;
                if (is_ac) { off = a * (-1) / h * m->stack_sign[inz]; dg = a * 1 / h * m->stack_sign[inz]; }
                else { off = a * (-1) / h * m->stack_epsn[inz] * EPSILON0; dg = a * 1 / h * m->stack_epsn[inz] * EPSILON0; }
            } else {
                if (is_ac) dg = fabs(a * 1 / h * m->stack_sign[inz]);
                else dg = fabs(a * 1 / h * m->stack_epsn[inz] * EPSILON0);
            }
            /* unordered_map accumulation in entry order (off-diagonal first) */
            if (nr + 2 > rowcap) { rowcap = rowcap ? rowcap * 2 : 64; row = (kv_t *)realloc(row, sizeof(kv_t) * (size_t)rowcap); }
            if (other >= 0) {
                if (pos[other] < 0) { pos[other] = nr; row[nr].col = other; row[nr].val = 0.0; nr++; }
                row[pos[other]].val += off;
            }
            if (pos[c] < 0) { pos[c] = nr; row[nr].col = c; row[nr].val = 0.0; nr++; }
            row[pos[c]].val += dg;
        }
        for (int64_t t = 0; t < nr; t++) pos[row[t].col] = -1;
        qsort(row, (size_t)nr, sizeof(kv_t), cmp_kv);
        for (int64_t t = 0; t < nr; t++) {
            if (!is_ac && !(fabs(row[t].val) > 1e-8)) continue;    /* fdtd.hpp:2852 */
            if (nnz == cap) { cap *= 2; A->col = (int64_t *)realloc(A->col, sizeof(int64_t) * (size_t)cap); A->val = (double *)realloc(A->val, sizeof(double) * (size_t)cap); }
            A->col[nnz] = row[t].col; A->val[nnz] = row[t].val; nnz++;
        }
        A->ptr[c + 1] = nnz;
    }
    free(row);
    free(pos);
    return 0;
}

int g2po_ad(const g2po_mesh *m, const g2po_v0 *v, g2po_csr *A) { return assemble_laplacian(m, v, 0, A); }
int g2po_ac(const g2po_mesh *m, const g2po_v0 *v, g2po_csr *A) { return assemble_laplacian(m, v, 1, A); }

/* ------------------------------------------ V0 products (mkl_sparse_d_mv, a14) */
/* y = V^T x over the column-major V0 COO (NON_TRANSPOSE on the CSR of V^T) */
static void v0t_mv(const g2po_v0 *v, int use_a, const double *x, double *y) {
    int64_t k = 0;
    for (int64_t c = 0; c < v->ncol; c++) {
        double s = 0.0;
        for (; k < v->nnz && v->col[k] == c; k++) s += (use_a ? v->aval[k] : v->val[k]) * x[v->row[k]];
        y[c] = s;
    }
}

/* y = V x (TRANSPOSE on the CSR of V^T), accumulated column by column */
static void v0_mv(const g2po_v0 *v, int use_a, const double *x, double *y, int64_t nedge) {
    memset(y, 0, sizeof(double) * (size_t)nedge);
    for (int64_t k = 0; k < v->nnz; k++) {
        double xi = 1.0 * x[v->col[k]];
        y[v->row[k]] += (use_a ? v->aval[k] : v->val[k]) * xi;
    }
}

static double freq_of(const g2po_mesh *m, int id) {
    /* fdtd.hpp:4319-4334 and print_z_V0's id==nfreq-1 branch (:4280-4283) */
    if (m->nfreq == 1) return m->freq_start * m->freq_unit;
    if (id == m->nfreq - 1) return m->freq_end * m->freq_unit;
    if (m->freq_scale == 1) return (m->freq_start + id * (m->freq_end - m->freq_start) / (m->nfreq - 1)) * m->freq_unit;
    return m->freq_start * m->freq_unit * pow(m->freq_end / m->freq_start, (id * 1.0 / (m->nfreq - 1)));
}

/* ---------------------------------------------------------- the V0 job
 * paraGenerator's default path (matrixCon.cpp:11-907 with SKIP_VH) split
 * into its assembly and, per port, its three solves (Ad, Ac, Ad), so that a
 * caller can run the ports of one job on several host threads: the ports
 * share only read-only data (V0 bases, Ad, Ac) and, without setup reuse,
 * each solve builds its own hierarchy as hypreSolve does. */
typedef struct {
    double *J, *y0d, *yd1, *yc, *yd2, *ydt, *bd, *bc, *crhs, *y0c;
    double *ydat;  /* V0da * y0d (the full-wave path's u0a) */
    int stage;     /* next stage to run: 0 first Ad solve, 1 Ac solve, 2 second Ad solve, 3 done */
    /* kept for the full-wave path (g2po_job_enable_vh): u0, u0a (2 columns
       over the non-PEC edges, real), yd (complex over all edges) and J */
    double *u0, *u0a, *yd_re, *yd_im, *Jkeep;
} port_state;

struct g2po_job {
    const g2po_mesh *m;
    dims_t d;
    int64_t *map_edge;
    uint8_t *pec_edge, *pec_node;
    g2po_v0 vd, vc;
    g2po_csr Ad, Ac;
    port_state *ps;
    double *zr, *zi;
    int keep_vh;                 /* keep each port's fields for the full-wave path */
    g2po_csr S;                  /* stiffness over the non-PEC edges (full-wave path) */
    int64_t *map_r;              /* mapEdgeR: non-PEC edge index -> edge */
    int64_t nr;                  /* N_edge - bden */
};

g2po_job *g2po_job_create(const g2po_mesh *m, g2po_para_stats *st) {
    double t0 = now_s();
    g2po_job *j = (g2po_job *)calloc(1, sizeof(*j));
    j->m = m;
    j->d = dims(m);
    memset(st, 0, sizeof(*st));
    j->map_edge = (int64_t *)malloc(sizeof(int64_t) * (size_t)j->d.N_edge);
    j->pec_edge = (uint8_t *)malloc((size_t)j->d.N_edge);
    j->pec_node = (uint8_t *)malloc((size_t)j->d.N_node);
    st->bden = g2po_index_maps(m, j->map_edge, j->pec_edge, j->pec_node);
    g2po_v0d(m, j->pec_node, &j->vd);
    g2po_ad(m, &j->vd, &j->Ad);
    g2po_v0c(m, j->pec_node, &j->vc);
    g2po_ac(m, &j->vc, &j->Ac);
    st->leng_v0d = j->vd.ncol; st->leng_v0c = j->vc.ncol;
    st->nnz_ad = j->Ad.ptr[j->Ad.n]; st->nnz_ac = j->Ac.ptr[j->Ac.n];
    j->ps = (port_state *)calloc((size_t)m->num_ports, sizeof(port_state));
    j->zr = (double *)calloc((size_t)m->num_ports * m->num_ports, sizeof(double));
    j->zi = (double *)calloc((size_t)m->num_ports * m->num_ports, sizeof(double));
    st->t_assembly = now_s() - t0;
    return j;
}

static void port_free_work(port_state *q) {
    free(q->J); free(q->y0d); free(q->yd1); free(q->yc); free(q->yd2); free(q->ydt); free(q->bd); free(q->bc);
    free(q->crhs); free(q->y0c); free(q->ydat);
    q->J = q->y0d = q->yd1 = q->yc = q->yd2 = q->ydt = q->bd = q->bc = q->crhs = q->y0c = q->ydat = NULL;
}

static void port_free(port_state *q) {
    port_free_work(q);
    free(q->u0); free(q->u0a); free(q->yd_re); free(q->yd_im); free(q->Jkeep);
    memset(q, 0, sizeof(*q));
}

/* The port's V0 fields the full-wave path reads (matrixCon.cpp:414-430,
 * 545-576): u0 and u0a, two unit columns over the non-PEC edges (the first
 * Ad solve's V0d and V0da products, then the second Ad and the Ac solves'
 * sums), and yd = (yd2 + yc) - i yd1 over all edges, with J. */
static void keep_vh_fields(struct g2po_job *j, port_state *q) {
    const int64_t ne = j->d.N_edge, nr = j->nr;
    double *yd2a = (double *)calloc((size_t)ne, sizeof(double)), *yca = (double *)calloc((size_t)ne, sizeof(double));
    v0_mv(&j->vd, 1, q->y0d, yd2a, ne);
    v0_mv(&j->vc, 1, q->y0c, yca, ne);
    double nn = 0, nna = 0;
    for (int64_t e = 0; e < ne; e++) { nn += q->yd1[e] * q->yd1[e]; nna += q->ydat[e] * q->ydat[e]; }
    nn = sqrt(nn);
    nna = sqrt(nna);
    q->u0 = (double *)calloc((size_t)(2 * nr), sizeof(double));
    q->u0a = (double *)calloc((size_t)(2 * nr), sizeof(double));
    for (int64_t i = 0; i < nr; i++) {
        q->u0[i] = q->yd1[j->map_r[i]] / nn;
        q->u0a[i] = q->ydat[j->map_r[i]] / nna;
    }
    nn = 0;
    nna = 0;
    for (int64_t e = 0; e < ne; e++) {
        nn += (q->yd2[e] + q->yc[e]) * (q->yd2[e] + q->yc[e]);
        nna += (yd2a[e] + yca[e]) * (yd2a[e] + yca[e]);
    }
    nn = sqrt(nn);
    nna = sqrt(nna);
    for (int64_t i = 0; i < nr; i++) {
        q->u0[nr + i] = (q->yd2[j->map_r[i]] + q->yc[j->map_r[i]]) / nn;
        q->u0a[nr + i] = (yd2a[j->map_r[i]] + yca[j->map_r[i]]) / nna;
    }
    q->yd_re = (double *)malloc(sizeof(double) * (size_t)ne);
    q->yd_im = (double *)malloc(sizeof(double) * (size_t)ne);
    for (int64_t e = 0; e < ne; e++) {
        q->yd_re[e] = (q->yd2[e] - 0.0) + q->yc[e];
        q->yd_im[e] = 0.0 - q->yd1[e];
    }
    q->Jkeep = q->J;
    q->J = NULL;
    free(yd2a);
    free(yca);
}

static void job_solve(const g2po_csr *A, g2po_amg_handle *H, const double *b, double *x,
                      const g2po_solver_opts *o, g2po_solve_stats *ss, double *t_setup) {
    double t = now_s();
    g2po_amg_handle *h = H ? H : g2po_amg_create(A, o);
    *t_setup = H ? 0.0 : now_s() - t;
    g2po_amg_solve(h, b, x, o, ss);
    if (!H) g2po_amg_destroy(h);
}

/* Runs port p's next stage; H is a prebuilt hierarchy for the stage's matrix
 * (Ad for stages 0 and 2, Ac for stage 1) or NULL for a fresh setup.  Stage 2
 * also writes the port's column of Z (Construct_Z_V0, fdtd.hpp:4173-4215). */
static int job_stage(g2po_job *j, int p, g2po_amg_handle *H, const g2po_solver_opts *o, g2po_solve_stats *ss,
                     double *t_setup) {
    const g2po_mesh *m = j->m;
    const dims_t d = j->d;
    const int64_t ne = d.N_edge;
    const int P = m->num_ports;
    port_state *q = &j->ps[p];
    const double omega = (2 * M_PI * m->freq_start * m->freq_unit);
    if (q->stage == 0) {
        q->J = (double *)calloc((size_t)ne, sizeof(double));
        q->bd = (double *)calloc((size_t)j->vd.ncol, sizeof(double));
        q->y0d = (double *)calloc((size_t)j->vd.ncol, sizeof(double));
        q->bc = (double *)calloc((size_t)j->vc.ncol, sizeof(double));
        q->crhs = (double *)calloc((size_t)j->vc.ncol, sizeof(double));
        q->y0c = (double *)calloc((size_t)j->vc.ncol, sizeof(double));
        q->ydt = (double *)calloc((size_t)ne, sizeof(double));
        q->yd1 = (double *)calloc((size_t)ne, sizeof(double));
        q->yc = (double *)calloc((size_t)ne, sizeof(double));
        q->yd2 = (double *)calloc((size_t)ne, sizeof(double));
        /* matrixCon.cpp:365-374 */
        for (int s = m->port_side_ptr[p]; s < m->port_side_ptr[p + 1]; s++)
            for (int64_t k = m->side_edge_ptr[s]; k < m->side_edge_ptr[s + 1]; k++)
                q->J[m->side_edges[k]] = m->side_dir[s];
        /* :384-392 */
        v0t_mv(&j->vd, 1, q->J, q->bd);
        for (int64_t i = 0; i < j->vd.ncol; i++) q->bd[i] *= -1.0;
        job_solve(&j->Ad, H, q->bd, q->y0d, o, ss, t_setup);
    } else if (q->stage == 1) {
        /* :401-412 */
        for (int64_t i = 0; i < j->vd.ncol; i++) q->y0d[i] /= omega;
        v0_mv(&j->vd, 0, q->y0d, q->ydt, ne);
        if (j->keep_vh) {
            q->ydat = (double *)calloc((size_t)ne, sizeof(double));
            v0_mv(&j->vd, 1, q->y0d, q->ydat, ne);
        }
        /* :436-461 */
        v0t_mv(&j->vc, 1, q->J, q->bc);
        for (int64_t i = 0; i < j->vc.ncol; i++) q->bc[i] *= -1.0;
        for (int64_t e = 0; e < ne; e++) {
            q->yd1[e] = q->ydt[e];
            q->ydt[e] *= -1.0 * (2 * M_PI * m->freq_start * m->freq_unit) * m->stack_epsn[e / d.L] * EPSILON0;
        }
        v0t_mv(&j->vc, 1, q->ydt, q->crhs);
        for (int64_t i = 0; i < j->vc.ncol; i++) q->bc[i] += q->crhs[i];
        /* :511 */
        job_solve(&j->Ac, H, q->bc, q->y0c, o, ss, t_setup);
    } else if (q->stage == 2) {
        /* :528-544 */
        v0_mv(&j->vc, 0, q->y0c, q->yc, ne);
        for (int64_t e = 0; e < ne; e++) q->ydt[e] = -q->yc[e] * m->stack_epsn[e / d.L] * EPSILON0;
        v0t_mv(&j->vd, 1, q->ydt, q->bd);
        job_solve(&j->Ad, H, q->bd, q->y0d, o, ss, t_setup);
        /* :553-584: yd = (yd2 + yc) - i*yd1 */
        v0_mv(&j->vd, 0, q->y0d, q->yd2, ne);
        /* Construct_Z_V0 (fdtd.hpp:4173-4215) */
        double cur = 0.0;
        for (int s = m->port_side_ptr[p]; s < m->port_side_ptr[p + 1]; s++) cur += m->side_area[s];
        for (int r = 0; r < P; r++) {
            int s = m->port_side_ptr[r];
            double re = 0.0, im = 0.0;
            for (int64_t k = m->side_edge_ptr[s]; k < m->side_edge_ptr[s + 1]; k++) {
                int64_t e = m->side_edges[k];
                int64_t rr = e % d.L;
                double leng;
                if (rr >= d.Ns) { int64_t inz = e / d.L; leng = m->zn[inz + 1] - m->zn[inz]; }
                else if (rr >= d.Ny * (d.Nx + 1)) { int64_t inx = (rr - d.Ny * (d.Nx + 1)) / (d.Ny + 1); leng = m->xn[inx + 1] - m->xn[inx]; }
                else { int64_t iny = rr % d.Ny; leng = m->yn[iny + 1] - m->yn[iny]; }
                double dir = m->side_dir[s] * 1.0;
                double yre = (q->yd2[e] - 0.0) + q->yc[e];
                double yim = 0.0 - q->yd1[e];
                re -= yre * leng * dir;
                im -= yim * leng * dir;
            }
            j->zr[r + (int64_t)P * p] = re / cur;
            j->zi[r + (int64_t)P * p] = im / cur;
        }
        if (j->keep_vh) keep_vh_fields(j, q);
        port_free_work(q);
    } else {
        return -1;
    }
    q->stage++;
    return 0;
}

int g2po_job_port_stage(g2po_job *j, int port, const g2po_solver_opts *o, g2po_solve_stats *ss, double *t_setup) {
    if (!j || port < 0 || port >= j->m->num_ports) return -1;
    double ts = 0.0;
    int rc = job_stage(j, port, NULL, o, ss, &ts);
    if (t_setup) *t_setup = ts;
    return rc;
}

/* print_z_V0 (fdtd.hpp:4249-4316): freq 0 as stored, others transposed with
   Im scaled by f0/f */
void g2po_job_z(const g2po_job *j, double *z_out) {
    const g2po_mesh *m = j->m;
    const int P = m->num_ports;
    for (int f = 0; f < m->nfreq; f++) {
        double fr = freq_of(m, f);
        for (int i = 0; i < P; i++)
            for (int k = 0; k < P; k++) {
                int64_t o0 = (int64_t)f * P * P;
                if (f == 0) {
                    z_out[2 * (o0 + k + (int64_t)i * P)] = j->zr[k + (int64_t)i * P];
                    z_out[2 * (o0 + k + (int64_t)i * P) + 1] = j->zi[k + (int64_t)i * P];
                } else {
                    z_out[2 * (o0 + i + (int64_t)k * P)] = j->zr[k + (int64_t)i * P] + 0.0;
                    z_out[2 * (o0 + i + (int64_t)k * P) + 1] = j->zi[k + (int64_t)i * P] * m->freq_start * m->freq_unit / fr;
                }
            }
    }
}

void g2po_job_destroy(g2po_job *j) {
    if (!j) return;
    g2po_csr_free(&j->S);
    free(j->map_r);
    for (int p = 0; p < j->m->num_ports; p++) port_free(&j->ps[p]);
    free(j->ps); free(j->zr); free(j->zi);
    g2po_v0_free(&j->vd); g2po_v0_free(&j->vc);
    g2po_csr_free(&j->Ad); g2po_csr_free(&j->Ac);
    free(j->map_edge); free(j->pec_edge); free(j->pec_node);
    free(j);
}

int g2po_para_generator(const g2po_mesh *m, const g2po_solver_opts *o, int max_ports,
                        double *z_out, g2po_para_stats *st) {
    g2po_job *j = g2po_job_create(m, st);
    double t1 = now_s();
    const int P = m->num_ports;
    const int np = (max_ports > 0 && max_ports < P) ? max_ports : P;
    g2po_amg_handle *Hd = NULL, *Hc = NULL;
    double t_setup = 0.0, ts = now_s();
    if (o->reuse_setup) { Hd = g2po_amg_create(&j->Ad, o); Hc = g2po_amg_create(&j->Ac, o); }
    t_setup += now_s() - ts;
    for (int p = 0; p < np; p++) {
        for (int stage = 0; stage < 3; stage++) {
            g2po_solve_stats ss;
            double t = now_s(), tsu = 0.0;
            job_stage(j, p, stage == 1 ? Hc : Hd, o, &ss, &tsu);
            t_setup += tsu;
            st->solves++; st->total_iterations += ss.iterations;
            if (ss.rel_residual > st->max_rel_residual) st->max_rel_residual = ss.rel_residual;
            if (st->solves <= 3) st->t_each[st->solves - 1] = now_s() - t;
            if (o->stop_after_solves > 0 && st->solves >= o->stop_after_solves) goto sampled;
        }
    }
sampled:
    g2po_job_z(j, z_out);
    st->t_setup = t_setup;
    st->t_solve = now_s() - t1 - t_setup;
    if (Hd) g2po_amg_destroy(Hd);
    if (Hc) g2po_amg_destroy(Hc);
    g2po_job_destroy(j);
    return 0;
}

/* ------------------------------------------------- the full-wave (Vh) path
 * The reference compiles it out (SKIP_VH, fdtd.hpp:76).  With it in,
 * paraGenerator runs find_Vh(1000) once (matrixCon.cpp:331-333) and, for
 * every port and frequency, corrects the V0 field by a Galerkin projection on
 * the Vh eigenmodes (matrixCon.cpp:609-805); the dense LAPACK calls go to
 * oracle/lapacke_shim.cpp. */
typedef struct { double re, im; } zc;
long long LAPACKE_dhseqr(int, char, char, long long, long long, long long, double *, long long, double *, double *,
                         double *, long long);
long long LAPACKE_dhsein(int, char, char, char, long long *, long long, const double *, long long, double *,
                         const double *, double *, long long, double *, long long, long long, long long *,
                         long long *, long long *);
long long LAPACKE_zcgesv(int, long long, long long, zc *, long long, long long *, zc *, long long, zc *, long long,
                         long long *);
long long LAPACKE_zgesv(int, long long, long long, zc *, long long, long long *, zc *, long long);

#define SIGMA_CU (5.8e+7)     /* fdtd.hpp:50, the Vh products' conductivity */

int g2po_job_enable_vh(g2po_job *j) {
    if (!j) return -1;
    j->keep_vh = 1;
    if (g2po_stiffness(j->m, j->map_edge, j->pec_edge, &j->S) != 0) return -1;
    j->nr = j->S.n;
    j->map_r = (int64_t *)malloc(sizeof(int64_t) * (size_t)(j->nr > 0 ? j->nr : 1));
    for (int64_t e = 0; e < j->d.N_edge; e++)
        if (j->map_edge[e] >= 0) j->map_r[j->map_edge[e]] = e;
    for (int64_t r = 0; r < j->nr; r++)
        if (j->S.ptr[r + 1] == j->S.ptr[r]) return -2;      /* every row of S has its diagonal */
    return 0;
}

int64_t g2po_job_nr(const g2po_job *j) { return j->nr; }

/* find_Vh(k) (fdtd.hpp:3577-3859): k Arnoldi steps (modified Gram-Schmidt)
 * on the 2N operator [[0, I], [-eps^-1 S / scale^2, -eps^-1 sigma / scale]],
 * the Hessenberg matrix's eigenvalues, right eigenvectors of those with
 * |Im| > 1e-6, and Vh = V(1:N, 1:k) * eigenvectors.  *vh: nr x mm complex,
 * column-major, (re, im) interleaved; malloc'd. */
int g2po_find_vh(g2po_job *jb, int k, double **vh_out, int64_t *mm_out) {
    const g2po_mesh *m = jb->m;
    const dims_t d = jb->d;
    const int64_t nr = jb->nr, n2 = 2 * nr;
    const double scale = 1.e+14;
    const g2po_csr *S = &jb->S;
    double *V = (double *)calloc((size_t)((k + 1) * n2), sizeof(double));
    double *w = (double *)calloc((size_t)n2, sizeof(double));
    double *H = (double *)calloc((size_t)k * k, sizeof(double));
    for (int64_t i = 0; i < n2; i++) V[i] = 1 / sqrt(2 * nr);
    for (int jj = 1; jj <= k; jj++) {
        const double *vp = V + (int64_t)(jj - 1) * n2;
        for (int64_t row = 0; row < nr; row++) {
            const int64_t e = jb->map_r[row];
            w[nr + row] = 0;
            w[row] = vp[nr + row];
            for (int64_t q = S->ptr[row]; q < S->ptr[row + 1]; q++)
                w[nr + row] += -S->val[q] * vp[S->col[q]] / (m->stack_epsn[e / d.L] * EPSILON0 * pow(scale, 2));
            if (m->mark_edge[e] != 0)
                w[nr + row] += -vp[nr + row] * m->stack_sign[e / d.L] / (m->stack_epsn[e / d.L] * EPSILON0 * scale);
        }
        double *hcol = H + (int64_t)(jj - 1) * k;
        for (int i = 0; i <= jj - 1; i++) {
            const double *vi = V + (int64_t)i * n2;
            for (int64_t in = 0; in < n2; in++) hcol[i] += vi[in] * w[in];
            for (int64_t in = 0; in < n2; in++) w[in] -= hcol[i] * vi[in];
        }
        double temp;
        if (jj == k) {
            temp = 0;
            for (int64_t i = 0; i < n2; i++) temp += pow(w[i], 2);
            temp = sqrt(temp);
        } else {
            for (int64_t i = 0; i < n2; i++) hcol[jj] += pow(w[i], 2);
            hcol[jj] = sqrt(hcol[jj]);
            temp = hcol[jj];
        }
        for (int64_t i = 0; i < n2; i++) V[(int64_t)jj * n2 + i] = w[i] / temp;
    }
    double *H1 = (double *)calloc((size_t)k * k, sizeof(double));
    for (int i = 0; i < k; i++)
        for (int c = 0; c < k; c++)
            if (i <= c + 1) H1[c * k + i] = H[c * k + i];
    double *wr = (double *)malloc(sizeof(double) * k), *wi = (double *)malloc(sizeof(double) * k);
    LAPACKE_dhseqr(102, 'E', 'N', k, 1, k, H, k, wr, wi, NULL, k);
    long long *select = (long long *)calloc((size_t)k, sizeof(long long));
    long long mm = 0;
    for (int i = 0; i < k; i++) {
        if (fabs(wi[i]) > 1e-6) { select[i] = 1; mm++; }
    }
    long long mret = 0;
    long long *ifaill = (long long *)calloc((size_t)(mm > 0 ? mm : 1), sizeof(long long));
    long long *ifailr = (long long *)calloc((size_t)(mm > 0 ? mm : 1), sizeof(long long));
    double *vr = (double *)calloc((size_t)(k * (mm > 0 ? mm : 1)), sizeof(double));
    LAPACKE_dhsein(102, 'R', 'Q', 'N', select, k, H1, k, wr, wi, NULL, k, vr, k, mm, &mret, ifaill, ifailr);
    zc *v = (zc *)calloc((size_t)(k * (mm > 0 ? mm : 1)), sizeof(zc));
    for (int i = 0; i < k; i++) {
        int64_t t = 0;
        for (int c = 0; c < k; c++)
            if (select[c] == 1) {
                v[t * k + i].re = vr[t * k + i];
                v[t * k + i].im = vr[(t + 1) * k + i];
                v[(t + 1) * k + i].re = vr[t * k + i];
                v[(t + 1) * k + i].im = -vr[(t + 1) * k + i];
                t += 2;
                c++;
            }
    }
    double *vh = (double *)malloc(sizeof(double) * (size_t)(2 * nr * (mm > 0 ? mm : 1)));
    for (int64_t i = 0; i < mm; i++)
        for (int64_t r = 0; r < nr; r++) {
            double re = 0, im = 0;
            for (int in = 0; in < k; in++) {
                re += V[(int64_t)in * n2 + r] * v[i * k + in].re;
                im += V[(int64_t)in * n2 + r] * v[i * k + in].im;
            }
            vh[2 * (i * nr + r)] = re;
            vh[2 * (i * nr + r) + 1] = im;
        }
    free(V); free(w); free(H); free(H1); free(wr); free(wi); free(select); free(ifaill); free(ifailr); free(vr);
    free(v);
    *vh_out = vh;
    *mm_out = mm;
    return 0;
}

/* matrix_multi (findVh.cpp:1205): 'T' gives conj(a)^T b, 'N' gives a b, for
 * column-major complex a (arow x acol) and b (brow x bcol). */
static void zmulti(char op, const zc *a, int64_t arow, int64_t acol, const zc *b, int64_t brow, int64_t bcol, zc *out) {
    if (op == 'T') {
        for (int64_t i = 0; i < acol; i++)
            for (int64_t c = 0; c < bcol; c++) {
                double re = 0, im = 0;
                for (int64_t r = 0; r < arow; r++) {
                    re = re + a[i * arow + r].re * b[c * brow + r].re + a[i * arow + r].im * b[c * brow + r].im;
                    im = im - a[i * arow + r].im * b[c * brow + r].re + a[i * arow + r].re * b[c * brow + r].im;
                }
                out[c * acol + i].re = re;
                out[c * acol + i].im = im;
            }
    } else {
        for (int64_t i = 0; i < arow; i++)
            for (int64_t c = 0; c < bcol; c++) {
                double re = 0, im = 0;
                for (int64_t r = 0; r < acol; r++) {
                    re = re + a[r * arow + i].re * b[c * brow + r].re - a[r * arow + i].im * b[c * brow + r].im;
                    im = im + a[r * arow + i].im * b[c * brow + r].re + a[r * arow + i].re * b[c * brow + r].im;
                }
                out[c * arow + i].re = re;
                out[c * arow + i].im = im;
            }
    }
}

/* (-w^2 D_eps + i w D_sig) on one complex entry of the non-PEC edge r, as the
 * Vh products write it (matrixCon.cpp:625-634): the layer index of edge e is
 * (e + N_edge_v) / L there, and sigma is SIGMA (fdtd.hpp:50). */
static zc diag_op(const g2po_job *jb, int64_t r, zc x, double freq) {
    const int64_t e = jb->map_r[r];
    const double eps = jb->m->stack_epsn[(e + jb->d.Nv) / jb->d.L];
    zc y;
    if (jb->m->mark_edge[e] != 0) {
        y.re = x.re * (-freq * freq * 4 * pow(M_PI, 2)) * eps * EPSILON0 - 2 * M_PI * freq * x.im * SIGMA_CU;
        y.im = x.re * (freq * 2 * M_PI) * SIGMA_CU - x.im * (freq * freq * 4 * pow(M_PI, 2)) * eps * EPSILON0;
    } else {
        y.re = x.re * (-freq * freq * 4 * pow(M_PI, 2)) * eps * EPSILON0;
        y.im = -x.im * (freq * freq * 4 * pow(M_PI, 2)) * eps * EPSILON0;
    }
    return y;
}

/* The Vh correction of every port at every frequency (matrixCon.cpp:609-805)
 * and Construct_Z_V0_Vh (fdtd.hpp:4133-4170).  Every port must have run its
 * three stages with g2po_job_enable_vh on.  z_vh[f][q + P p] (complex,
 * interleaved): Construct_Z_V0_Vh into zeros.  z_ref: sys->x as the
 * reference leaves it with PRINT_V0_Vh_Z_PARAM, where the first frequency's
 * entries start from Construct_Z_V0's V0 values instead of zero. */
int g2po_job_vh_z(g2po_job *jb, const double *vh_in, int64_t mm, double *z_vh, double *z_ref) {
    const g2po_mesh *m = jb->m;
    const dims_t d = jb->d;
    const int64_t nr = jb->nr;
    const int P = m->num_ports;
    const zc *Vh0 = (const zc *)vh_in;
    const g2po_csr *S = &jb->S;
    zc *V_re2 = (zc *)malloc(sizeof(zc) * (size_t)(nr * mm)), *Vh = (zc *)malloc(sizeof(zc) * (size_t)(nr * mm));
    zc *tmp = (zc *)malloc(sizeof(zc) * (size_t)(nr * (mm > 2 ? mm : 2)));
    zc *y_re = (zc *)calloc((size_t)(2 * mm), sizeof(zc)), *y_new = (zc *)calloc((size_t)(2 * mm), sizeof(zc));
    zc *m_new = (zc *)calloc((size_t)(nr * mm), sizeof(zc)), *m_h = (zc *)calloc((size_t)(mm * mm), sizeof(zc));
    zc *rhs_h = (zc *)calloc((size_t)mm, sizeof(zc)), *rhs_h0 = (zc *)calloc((size_t)mm, sizeof(zc));
    zc *Jc = (zc *)calloc((size_t)nr, sizeof(zc)), *y_h = (zc *)calloc((size_t)nr, sizeof(zc));
    zc *final_x = (zc *)malloc(sizeof(zc) * (size_t)nr);
    zc u0[2], tmp4[4];
    long long ipiv2[2], iter = 0;
    long long *ipiv = (long long *)malloc(sizeof(long long) * (size_t)(mm > 0 ? mm : 1));
    memset(z_vh, 0, sizeof(double) * 2 * (size_t)m->nfreq * P * P);
    memset(z_ref, 0, sizeof(double) * 2 * (size_t)m->nfreq * P * P);
    for (int p = 0; p < P; p++) {
        const port_state *q = &jb->ps[p];
        if (!q->u0) return -1;
        zc *U0 = (zc *)calloc((size_t)(2 * nr), sizeof(zc)), *U0a = (zc *)calloc((size_t)(2 * nr), sizeof(zc));
        for (int64_t i = 0; i < 2 * nr; i++) { U0[i].re = q->u0[i]; U0a[i].re = q->u0a[i]; }
        /* the reference's first frequency starts from Construct_Z_V0 */
        for (int r = 0; r < P; r++) {
            z_ref[2 * (r + (int64_t)P * p)] = jb->zr[r + (int64_t)P * p];
            z_ref[2 * (r + (int64_t)P * p) + 1] = jb->zi[r + (int64_t)P * p];
        }
        for (int fi = 0; fi < m->nfreq; fi++) {
            const double freq = freq_of(m, fi);
            /* Vh = Vh - u0 ((u0a' A u0) \\ (u0a' A Vh)) */
            for (int64_t r = 0; r < nr; r++)
                for (int64_t c = 0; c < mm; c++) V_re2[c * nr + r] = diag_op(jb, r, Vh0[c * nr + r], freq);
            zmulti('T', U0a, nr, 2, V_re2, nr, mm, y_re);
            for (int64_t r = 0; r < nr; r++)
                for (int c = 0; c < 2; c++) tmp[c * nr + r] = diag_op(jb, r, U0[c * nr + r], freq);
            zmulti('T', U0a, nr, 2, tmp, nr, 2, tmp4);
            LAPACKE_zcgesv(102, 2, mm, tmp4, 2, ipiv2, y_re, 2, y_new, 2, &iter);
            zmulti('N', U0, nr, 2, y_new, 2, mm, m_new);
            for (int64_t r = 0; r < nr; r++)
                for (int64_t c = 0; c < mm; c++) {
                    Vh[c * nr + r].re = Vh0[c * nr + r].re - m_new[c * nr + r].re;
                    Vh[c * nr + r].im = Vh0[c * nr + r].im - m_new[c * nr + r].im;
                }
            /* Vh' (S - w^2 D_eps + i w D_sig) Vh */
            for (int64_t c = 0; c < mm; c++) {
                zc *t = tmp + c * nr;
                for (int64_t r = 0; r < nr; r++) t[r].re = t[r].im = 0;
                for (int64_t r = 0; r < nr; r++)
                    for (int64_t qq = S->ptr[r]; qq < S->ptr[r + 1]; qq++) {
                        t[r].re += S->val[qq] * Vh[c * nr + S->col[qq]].re;
                        t[r].im += S->val[qq] * Vh[c * nr + S->col[qq]].im;
                    }
                for (int64_t r = 0; r < nr; r++) {
                    const int64_t e = jb->map_r[r];
                    const double eps = m->stack_epsn[(e + d.Nv) / d.L];
                    const zc x = Vh[c * nr + r];
                    if (m->mark_edge[e] != 0) {
                        t[r].re += -pow(freq * 2 * M_PI, 2) * eps * EPSILON0 * x.re - freq * 2 * M_PI * SIGMA_CU * x.im;
                        t[r].im += -pow(freq * 2 * M_PI, 2) * eps * EPSILON0 * x.im + freq * 2 * M_PI * SIGMA_CU * x.re;
                    } else {
                        t[r].re += -pow(freq * 2 * M_PI, 2) * eps * EPSILON0 * x.re;
                        t[r].im += -pow(freq * 2 * M_PI, 2) * eps * EPSILON0 * x.im;
                    }
                }
            }
            zmulti('T', Vh, nr, mm, tmp, nr, mm, m_h);
            /* -i w Vh' J */
            memset(Jc, 0, sizeof(zc) * (size_t)nr);
            for (int64_t e = 0; e < d.N_edge; e++)
                if (q->Jkeep[e] != 0) Jc[jb->map_edge[e]].im = -1 * freq * 2 * M_PI;
            zmulti('T', Vh, nr, mm, Jc, nr, 1, rhs_h);
            /* minus Vh' A u, u the V0 field at this frequency */
            const double fS = m->freq_start, fU = m->freq_unit;
            for (int64_t r = 0; r < nr; r++) {
                const int64_t e = jb->map_r[r];
                const double eps = m->stack_epsn[(e + d.Nv) / d.L];
                const double yr = q->yd_re[e], yi = q->yd_im[e];
                if (m->mark_edge[e] != 0) {
                    tmp[r].re = -pow(freq * 2 * M_PI, 2) * eps * EPSILON0 * yr - freq * 2 * M_PI * SIGMA_CU * yi * fS * fU / freq;
                    tmp[r].im = freq * 2 * M_PI * SIGMA_CU * yr - pow(freq * 2 * M_PI, 2) * eps * EPSILON0 * yi * fS * fU / freq;
                } else {
                    tmp[r].re = -pow(freq * 2 * M_PI, 2) * eps * EPSILON0 * yr;
                    tmp[r].im = -pow(freq * 2 * M_PI, 2) * eps * EPSILON0 * yi * fS * fU / freq;
                }
            }
            zmulti('T', Vh, nr, mm, tmp, nr, 1, rhs_h0);
            for (int64_t c = 0; c < mm; c++) {
                rhs_h[c].re = rhs_h[c].re - rhs_h0[c].re;
                rhs_h[c].im = rhs_h[c].im - rhs_h0[c].im;
            }
            LAPACKE_zgesv(102, mm, 1, m_h, mm, ipiv, rhs_h, mm);
            zmulti('N', Vh, nr, mm, rhs_h, mm, 1, y_h);
            for (int64_t r = 0; r < nr; r++) {
                const int64_t e = jb->map_r[r];
                final_x[r].re = q->yd_re[e] + y_h[r].re + 0.0;
                final_x[r].im = q->yd_im[e] * m->freq_start * m->freq_unit / freq + y_h[r].im;
            }
            /* Construct_Z_V0_Vh (fdtd.hpp:4133-4170) */
            double cur = 0.;
            for (int s = m->port_side_ptr[p]; s < m->port_side_ptr[p + 1]; s++) cur += m->side_area[s];
            for (int r = 0; r < P; r++) {
                const int s = m->port_side_ptr[r];
                double *zv = z_vh + 2 * ((int64_t)fi * P * P + r + (int64_t)P * p);
                double *zf = z_ref + 2 * ((int64_t)fi * P * P + r + (int64_t)P * p);
                for (int64_t kk = m->side_edge_ptr[s]; kk < m->side_edge_ptr[s + 1]; kk++) {
                    const int64_t e = m->side_edges[kk], rr = e % d.L;
                    double leng;
                    if (rr >= d.Ns) { int64_t inz = e / d.L; leng = m->zn[inz + 1] - m->zn[inz]; }
                    else if (rr >= d.Ny * (d.Nx + 1)) { int64_t inx = (rr - d.Ny * (d.Nx + 1)) / (d.Ny + 1); leng = m->xn[inx + 1] - m->xn[inx]; }
                    else { int64_t iny = rr % d.Ny; leng = m->yn[iny + 1] - m->yn[iny]; }
                    const double dir = m->side_dir[s] * 1.0;
                    const zc fx = final_x[jb->map_edge[e]];
                    zv[0] -= fx.re * leng * dir;
                    zv[1] -= fx.im * leng * dir;
                    zf[0] -= fx.re * leng * dir;
                    zf[1] -= fx.im * leng * dir;
                }
                zv[0] /= cur; zv[1] /= cur;
                zf[0] /= cur; zf[1] /= cur;
            }
        }
        free(U0); free(U0a);
    }
    (void)u0;
    free(V_re2); free(Vh); free(tmp); free(y_re); free(y_new); free(m_new); free(m_h); free(rhs_h); free(rhs_h0);
    free(Jc); free(y_h); free(final_x); free(ipiv);
    return 0;
}
