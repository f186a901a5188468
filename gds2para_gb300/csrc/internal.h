// Internal handle layouts (not part of the ABI).
#pragma once
#include <vector>
#include "common.cuh"

namespace g2p {

constexpr uint8_t kSellLong = 255;   // rlen of a row served by the long-row kernels

// Device CSR with int64 row offsets and int32 columns, plus an optional
// sliced-ELL copy of its short rows for the SpMM: slices of 32 rows whose
// entries are stored column by column (entry j of row 32 s + t at
// sptr[s] + 32 j + t), rlen[i] the row's entry count or kSellLong.  When
// ell_w > 0 every slice is ell_w wide (sptr[s] = 32 ell_w s) and the unused
// slots hold (column = the row, value = 0), so the kernel needs neither
// sptr nor rlen.
template <class T>
struct Csr {
    int64_t n = 0, m = 0, nnz = 0;
    int64_t *ptr = nullptr;
    int32_t *col = nullptr;
    T *val = nullptr;
    int64_t *sptr = nullptr;
    int32_t *scol = nullptr;
    T *sval = nullptr;
    uint8_t *rlen = nullptr;
    int64_t short_nnz = 0, sell_slots = 0;
    int32_t ell_w = 0;           // > 0: every slice has this width, padded with (row, 0)
    void release_sell(cudaStream_t s) {
        dfree(sptr, s); dfree(scol, s); dfree(sval, s); dfree(rlen, s);
        short_nnz = sell_slots = 0;
        ell_w = 0;
    }
    void release(cudaStream_t s) {
        dfree(ptr, s); dfree(col, s); dfree(val, s);
        release_sell(s);
        n = m = nnz = 0;
    }
};

// One V0 basis: column-major (CSR over columns, entries in the reference's
// COO order) plus the per-edge view used by V0*y (at most two entries per
// edge, ascending column).
struct V0Basis {
    int64_t ncol = 0, nnz = 0;
    int64_t *cptr = nullptr;   // [ncol+1]
    int32_t *cedge = nullptr;  // [nnz] original edge index
    double *cval = nullptr;    // [nnz] +-1/h
    double *caval = nullptr;   // [nnz] a-values
    int32_t *map = nullptr;    // [N_node] column+1 or 0
    // per-edge view: up to two (column, val, aval) per edge
    int32_t *ecol = nullptr;   // [2*N_edge], -1 when absent
    double *eval = nullptr;    // [2*N_edge]
    double *eaval = nullptr;   // [2*N_edge]
    void release(cudaStream_t s) {
        dfree(cptr, s); dfree(cedge, s); dfree(cval, s); dfree(caval, s); dfree(map, s);
        dfree(ecol, s); dfree(eval, s); dfree(eaval, s);
        ncol = nnz = 0;
    }
};

// A Laplacian whose ordered conductor sums still run on the side stream.
struct LapPending;

// The matrix-free curl-curl stencil of a mesh's S (stencil.cu).
struct CurlStencil;
void stencil_release(CurlStencil *st, cudaStream_t s);
g2p_status stencil_build(g2p_mesh *m, CurlStencil **out);
g2p_status stencil_apply(g2p_mesh *m, CurlStencil *st, const double *x, double *y, cudaStream_t s);
g2p_status stencil_check(CurlStencil *st, cudaStream_t s);

// The full-wave (Vh) state of a mesh: Vh and, while the V0 path runs for it,
// the ports' V0 field directions (fullwave.cu).
struct FullWave;
void fullwave_release(FullWave *fw, cudaStream_t s);
bool fullwave_active(const FullWave *fw);
g2p_status fullwave_keep_ports(g2p_mesh *m, int p0, int kk, const double *yd1, const double *ydat, const double *yd2,
                               const double *yc, const double *yd2a, const double *yca);

struct Constants {
    double mu, eps0;
};

}  // namespace g2p

struct g2p_mesh {
    g2p::Dims d;
    cudaStream_t stream = nullptr;
    int device = 0;
    g2p::Constants k;
    // geometry and materials (device)
    double *xn = nullptr, *yn = nullptr, *zn = nullptr;
    double *dxa = nullptr, *dya = nullptr, *dza = nullptr;    // dual lengths (generateStiff.cpp:250-267)
    double *epsn = nullptr, *sign = nullptr;
    int32_t *mark_node = nullptr, *mark_edge = nullptr;
    int64_t num_cdt = 0;
    int32_t *mark_port = nullptr;
    uint8_t *cdt_return = nullptr;
    // host copies of small inputs
    std::vector<double> h_xn, h_yn, h_zn, h_epsn, h_sign;
    std::vector<int32_t> h_mark_port;
    int32_t num_ports = 0;
    std::vector<int32_t> port_side_ptr;
    std::vector<int64_t> side_edge_ptr, side_edges;
    std::vector<double> side_area;
    std::vector<int32_t> side_dir;
    double freq_start = 0, freq_end = 0, freq_unit = 1;
    int32_t nfreq = 1, freq_scale = 1;
    // index maps
    bool maps_done = false;
    uint8_t *pec_edge = nullptr, *pec_node = nullptr;
    int32_t *map_edge = nullptr;
    int64_t bden = 0;
    // stiffness
    bool stiff_done = false;
    g2p::Csr<double> S;
    // V0 bases and Laplacians
    bool v0_done = false;
    g2p::LapPending *ad_pending = nullptr;   // Ad's long rows still summing on `side`
    cudaStream_t side = nullptr;
    double *v0_tab = nullptr;      // per-line quotient tables of the V0 entries
    g2p::V0Basis v0d, v0c;
    g2p::Csr<double> Ad, Ac;
    // full-wave mode (g2p_find_vh) and the matrix-free S it applies
    g2p::FullWave *fw = nullptr;
    g2p::CurlStencil *stencil = nullptr;
    // scratch for scans
    int64_t *scan_work = nullptr;
    int64_t scan_work_n = 0;
};
