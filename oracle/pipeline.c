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
    int stage;     /* next stage to run: 0 first Ad solve, 1 Ac solve, 2 second Ad solve, 3 done */
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

static void port_free(port_state *q) {
    free(q->J); free(q->y0d); free(q->yd1); free(q->yc); free(q->yd2); free(q->ydt); free(q->bd); free(q->bc);
    free(q->crhs); free(q->y0c);
    memset(q, 0, sizeof(*q));
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
        port_free(q);
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
