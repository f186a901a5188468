// Network parameters after the extraction: convertParam (Z, Y and S
// matrices per frequency, src/solnoutclass.hpp:1456-1610) as one GPU block per
// frequency, and the Touchstone 2.0 and CITIfile writers (dumpTouchstone,
// dumpCITI, src/solnoutclass.hpp:6040-6235).
//
// Matrices are P x P complex per frequency, stored as the reference's
// saveNetworkParam reads sys->x: entry (i, j) of frequency f at
// (f * P + i) * P + j, as interleaved (re, im) doubles.
#include <algorithm>
#include <cmath>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <string>
#include <vector>

#include "common.cuh"

using namespace g2p;

namespace g2p {
namespace {

constexpr int kMaxNetPorts = 64;

struct Cx {
    double re, im;
};
__device__ __forceinline__ Cx cadd(Cx a, Cx b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ Cx csub(Cx a, Cx b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ Cx cmul(Cx a, Cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ Cx cdiv(Cx a, Cx b) {
    const double d = b.re * b.re + b.im * b.im;
    return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
__device__ __forceinline__ double cabs2(Cx a) { return a.re * a.re + a.im * a.im; }

// In-place inverse of the n x n matrix m (row-major, shared memory) by
// Gauss-Jordan with partial pivoting; inv receives the result.
__device__ void cinverse(Cx *m, Cx *inv, int n, int *singular) {
    __shared__ int piv;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) inv[t] = {(t / n == t % n) ? 1.0 : 0.0, 0.0};
    __syncthreads();
    for (int k = 0; k < n; k++) {
        if (threadIdx.x == 0) {
            int p = k;
            double best = cabs2(m[k * n + k]);
            for (int r = k + 1; r < n; r++)
                if (cabs2(m[r * n + k]) > best) { best = cabs2(m[r * n + k]); p = r; }
            piv = p;
            if (best == 0.0) *singular = 1;
        }
        __syncthreads();
        const int p = piv;
        if (p != k)
            for (int j = threadIdx.x; j < n; j += blockDim.x) {
                Cx t = m[k * n + j]; m[k * n + j] = m[p * n + j]; m[p * n + j] = t;
                t = inv[k * n + j]; inv[k * n + j] = inv[p * n + j]; inv[p * n + j] = t;
            }
        __syncthreads();
        const Cx d = m[k * n + k];
        __syncthreads();
        for (int j = threadIdx.x; j < n; j += blockDim.x) {
            m[k * n + j] = cdiv(m[k * n + j], d);
            inv[k * n + j] = cdiv(inv[k * n + j], d);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
            const int r = t / n, j = t % n;
            if (r == k) continue;
            const Cx f = m[r * n + k];
            if (j != k) m[r * n + j] = csub(m[r * n + j], cmul(f, m[k * n + j]));
            inv[r * n + j] = csub(inv[r * n + j], cmul(f, inv[k * n + j]));
        }
        __syncthreads();
        for (int r = threadIdx.x; r < n; r += blockDim.x)
            if (r != k) m[r * n + k] = {0.0, 0.0};
        __syncthreads();
    }
}

// One frequency per block.  mode: 0 inverse (Z <-> Y); 1 Z -> S and 2 Y -> S
// (S = (L)(R)^-1 with L, R from the scaled matrix and the identity);
// 3 S -> Y and 4 S -> Z (D (I -/+ S)(I +/- S)^-1 D).
__global__ void k_convert(int n, const double *in, double *out, const double *droot, int mode, int *singular) {
    extern __shared__ Cx sh[];
    Cx *a = sh, *b = sh + n * n, *w = sh + 2 * n * n;
    const int64_t base = (int64_t)blockIdx.x * n * n;
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int i = t / n, j = t % n;
        Cx v = {in[2 * (base + t)], in[2 * (base + t) + 1]};
        const Cx one = {(i == j) ? 1.0 : 0.0, 0.0};
        if (mode == 0) {
            a[t] = v;
        } else if (mode == 1 || mode == 2) {
            // scaled matrix D M D with D = diag(sqrt(1 / Zs)) (Z) or diag(sqrt(Zs)) (Y)
            const Cx sc = {v.re * droot[i] * droot[j], v.im * droot[i] * droot[j]};
            if (mode == 1) { w[t] = csub(sc, one); a[t] = cadd(sc, one); }      // (DZD - I)(DZD + I)^-1
            else { w[t] = csub(one, sc); a[t] = cadd(one, sc); }                // (I - DYD)(I + DYD)^-1
        } else if (mode == 3) {
            w[t] = csub(one, v); a[t] = cadd(one, v);                          // D (I - S)(I + S)^-1 D
        } else {
            w[t] = cadd(one, v); a[t] = csub(one, v);                          // D (I + S)(I - S)^-1 D
        }
    }
    __syncthreads();
    cinverse(a, b, n, singular);
    // b = inverse; result = w * b (then scaled for modes 3, 4), or b itself
    for (int t = threadIdx.x; t < n * n; t += blockDim.x) {
        const int i = t / n, j = t % n;
        Cx r;
        if (mode == 0) {
            r = b[t];
        } else {
            r = {0.0, 0.0};
            for (int q = 0; q < n; q++) r = cadd(r, cmul(w[i * n + q], b[q * n + j]));
            if (mode >= 3) r = {r.re * droot[i] * droot[j], r.im * droot[i] * droot[j]};
        }
        out[2 * (base + t)] = r.re;
        out[2 * (base + t) + 1] = r.im;
    }
}

std::string timestamp(const char *fmt) {
    char buf[80];
    const time_t now = time(nullptr);
    struct tm tmv;
    localtime_r(&now, &tmv);
    strftime(buf, sizeof buf, fmt, &tmv);
    return buf;
}

// Spaces after a column label: the reference's width minus the extra digits
// of the indices, never negative (the reference's fill would throw from 50
// ports on).
std::string pad(int width, int i, int j) { return std::string((size_t)std::max(0, width - i / 10 - j / 10), ' '); }

}  // namespace
}  // namespace g2p

extern "C" g2p_status g2p_convert_param(char from, char to, int32_t nports, int32_t nfreq, const double *z_source,
                                        const double *in, double *out) {
    if (nports < 1 || nports > kMaxNetPorts || nfreq < 1 || !in || !out ||
        !(from == 'Z' || from == 'Y' || from == 'S') || !(to == 'Z' || to == 'Y' || to == 'S')) {
        set_last_message("g2p_convert_param: parameters Z, Y or S, 1..%d ports, nfreq >= 1", kMaxNetPorts);
        return G2P_ERR_INVALID;
    }
    const int64_t total = 2LL * nfreq * nports * nports;
    if (from == to) {
        if (out != in) G2P_CUDA(cudaMemcpy(out, in, sizeof(double) * total, cudaMemcpyDefault));
        return G2P_OK;
    }
    int mode;
    if ((from == 'Z' && to == 'Y') || (from == 'Y' && to == 'Z')) mode = 0;
    else if (from == 'Z') mode = 1;      // Z -> S
    else if (from == 'Y') mode = 2;      // Y -> S
    else if (to == 'Y') mode = 3;        // S -> Y
    else mode = 4;                       // S -> Z
    std::vector<double> root(nports, 1.0);
    if (mode != 0) {
        if (!z_source) { set_last_message("g2p_convert_param: S conversions need the port impedances"); return G2P_ERR_INVALID; }
        std::vector<double> zs(nports);
        G2P_CUDA(cudaMemcpy(zs.data(), z_source, sizeof(double) * nports, cudaMemcpyDefault));
        for (int i = 0; i < nports; i++) {
            if (!(zs[i] > 0)) { set_last_message("g2p_convert_param: port impedances must be positive"); return G2P_ERR_INVALID; }
            // Z -> S and S -> Y use sqrt(1 / Zs); Y -> S and S -> Z use sqrt(Zs)
            root[i] = (mode == 1 || mode == 3) ? std::sqrt(1.0 / zs[i]) : std::sqrt(zs[i]);
        }
    }
    cudaStream_t s;
    G2P_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    double *d_in = nullptr, *d_out = nullptr, *d_root = nullptr;
    int *d_sing = nullptr;
    auto run = [&]() -> g2p_status {
        G2P_TRY(dalloc(&d_in, total, s));
        G2P_TRY(dalloc(&d_out, total, s));
        G2P_TRY(dalloc(&d_root, nports, s));
        G2P_TRY(dalloc(&d_sing, 1, s));
        G2P_CUDA(cudaMemcpyAsync(d_in, in, sizeof(double) * total, cudaMemcpyDefault, s));
        G2P_CUDA(cudaMemcpyAsync(d_root, root.data(), sizeof(double) * nports, cudaMemcpyHostToDevice, s));
        G2P_CUDA(cudaMemsetAsync(d_sing, 0, sizeof(int), s));
        // three working matrices; the opt-in limit also covers the kernel's
        // own static shared memory beyond the default 48 KB
        const size_t shm = 3 * sizeof(Cx) * nports * nports;
        G2P_CUDA(cudaFuncSetAttribute(k_convert, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
        (kbegin("k_convert", s), k_convert<<<(unsigned)nfreq, 256, shm, s>>>(nports, d_in, d_out, d_root, mode, d_sing), kend(s));
        G2P_CUDA(cudaGetLastError());
        int sing = 0;
        G2P_CUDA(cudaMemcpyAsync(&sing, d_sing, sizeof(int), cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double) * total, cudaMemcpyDefault, s));
        G2P_CUDA(cudaStreamSynchronize(s));
        if (sing) { set_last_message("g2p_convert_param: singular matrix"); return G2P_ERR_INVALID; }
        return G2P_OK;
    };
    g2p_status st = run();
    dfree(d_in, s); dfree(d_out, s); dfree(d_root, s); dfree(d_sing, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return st;
}

// dumpTouchstone (src/solnoutclass.hpp:6118-6226).  All arrays are host
// memory; the matrices are in the reference's sys->x order.
extern "C" g2p_status g2p_write_touchstone(const char *path, char param, int32_t nports, int32_t nfreq,
                                           const double *freqs, const double *z_source, const double *p,
                                           const char *design) {
    if (!path || nports < 1 || nfreq < 1 || !freqs || !z_source || !p) {
        set_last_message("g2p_write_touchstone: invalid argument");
        return G2P_ERR_INVALID;
    }
    try {
        std::ofstream o(path);
        if (!o.is_open()) { set_last_message("g2p_write_touchstone: cannot open %s", path); return G2P_ERR_INVALID; }
        const int n = nports;
        o << "[Version] 2.0" << std::endl;
        o << "# Hz " << param << " RI R " << z_source[0] << std::endl;
        o << "[Number of Ports] " << n << std::endl;
        if (n == 2) o << "[Two-Port Data Order] 12_21" << std::endl;
        o << "[Number of Frequencies] " << nfreq << std::endl;
        o << "[Reference]" << std::endl;
        for (int q = 0; q < n; q++) o << z_source[q] << " ";
        o << std::endl << "[Matrix Format] Full" << std::endl;
        o << "! Date/Time " << timestamp("%Y-%m-%d %H:%M:%S") << std::endl;
        o << "! Name " << (design ? design : "") << std::endl;
        o << "! Provider: DARPA ERI IDEA/POSH Contributors" << std::endl;
        o << "! Program: Xyce Writer from DARPA ERI" << std::endl;
        o << "! Author: Purdue University" << std::endl;
        o << "[Network Data] " << std::endl;
        // column legend: at most four entries per line for more than two ports
        o << "!freq         ";
        for (int i = 0; i < n; i++) {
            for (int j = 0; j < n; j++) {
                if (n > 2 && i > 0 && j == 0)
                    o << "!Re" << param << i + 1 << "," << j + 1 << pad(7, i, j);
                else
                    o << "Re" << param << i + 1 << "," << j + 1 << pad(8, i, j);
                o << "Im" << param << i + 1 << "," << j + 1 << pad(8, i, j);
                if ((j + 1) % 4 == 0 && j + 1 != n && n > 2) o << std::endl << "!" << std::string(13, ' ');
            }
            if (n > 2) o << std::endl;
        }
        o << std::endl;
        for (int fi = 0; fi < nfreq; fi++) {
            o << std::left << std::setw(13) << std::setprecision(7) << freqs[fi] << " ";
            for (int i = 0; i < n; i++) {
                for (int j = 0; j < n; j++) {
                    const size_t t = 2 * (((size_t)fi * n + i) * n + j);
                    o << std::left << std::setw(13) << std::setprecision(7) << p[t] << " ";
                    o << std::left << std::setw(13) << std::setprecision(7) << p[t + 1] << " ";
                    if ((j + 1) % 4 == 0 && j + 1 != n && n > 2) o << std::endl << std::string(14, ' ');
                }
                if (n > 2) o << " ! row " << i + 1 << std::endl;
            }
            if (n <= 2) o << std::endl;
        }
        o << "[End]" << std::endl;
        o.close();
        if (o.fail()) { set_last_message("g2p_write_touchstone: write to %s failed", path); return G2P_ERR_INVALID; }
    } catch (const std::exception &e) {
        set_last_message("g2p_write_touchstone: %s", e.what());
        return G2P_ERR_INVALID;
    }
    return G2P_OK;
}

// dumpCITI (src/solnoutclass.hpp:6040-6115).  All arrays are host memory.
extern "C" g2p_status g2p_write_citi(const char *path, char param, int32_t nports, int32_t nfreq, const double *freqs,
                                     const double *p, const char *design) {
    if (!path || nports < 1 || nfreq < 1 || !freqs || !p) {
        set_last_message("g2p_write_citi: invalid argument");
        return G2P_ERR_INVALID;
    }
    try {
        std::ofstream o(path);
        if (!o.is_open()) { set_last_message("g2p_write_citi: cannot open %s", path); return G2P_ERR_INVALID; }
        std::string name = design ? design : "";
        for (auto &c : name) c = (char)toupper((unsigned char)c);
        const int n = nports;
        o << "CITIFILE A.01.01" << std::endl;
        o << "CONSTANT TIME " << timestamp("%Y %m %d %H %M %S") << std::endl;
        o << "NAME " << name << std::endl;
        o << "VAR FREQ MAG " << nfreq << std::endl;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) o << "DATA " << param << "[" << i + 1 << "," << j + 1 << "] RI" << std::endl;
        o << "VAR_LIST_BEGIN" << std::endl;
        for (int fi = 0; fi < nfreq; fi++) o << std::left << std::setw(13) << std::setprecision(7) << freqs[fi] << std::endl;
        o << "VAR_LIST_END" << std::endl;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                o << "BEGIN" << std::endl;
                for (int fi = 0; fi < nfreq; fi++) {
                    const size_t t = 2 * (((size_t)fi * n + i) * n + j);
                    o << std::right << std::setw(13) << std::setprecision(7) << p[t] << "," << std::left
                      << std::setw(13) << std::setprecision(7) << p[t + 1] << std::endl;
                }
                o << "END" << std::endl;
            }
        o.close();
        if (o.fail()) { set_last_message("g2p_write_citi: write to %s failed", path); return G2P_ERR_INVALID; }
    } catch (const std::exception &e) {
        set_last_message("g2p_write_citi: %s", e.what());
        return G2P_ERR_INVALID;
    }
    return G2P_OK;
}

namespace g2p {
namespace {

// The nodal conductance and capacitance matrices the reference's Xyce and
// SPEF writers print (row-major n x n), symmetrised as makeCSym/makeGSym do
// (src/solnoutclass.hpp:1319-1390): a matrix that is not approximately
// symmetric in Eigen's sense (|A - A^T|^2 <= 1e-24 min(|A|^2, |A^T|^2)) is
// replaced by (A + A^T) * 0.5.
struct Nodal {
    int n;
    std::vector<double> g, c;
    std::vector<double> g_ground, c_ground;    // row sums (getGNodeGround / getCNodeGround)
    double g_total = 0, c_total = 0;           // upper-triangle sums (getGTotal / getCTotal)
};

void symmetrise(std::vector<double> &a, int n) {
    double d2 = 0, na = 0, nt = 0;
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
            const double x = a[(size_t)i * n + j], y = a[(size_t)j * n + i];
            d2 += (x - y) * (x - y);
            na += x * x;
            nt += y * y;
        }
    const double prec = 1e-12;
    if (d2 <= prec * prec * std::min(na, nt)) return;
    std::vector<double> s(a.size());
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) s[(size_t)i * n + j] = (a[(size_t)i * n + j] + a[(size_t)j * n + i]) * 0.5;
    a.swap(s);
}

Nodal nodal(int n, const double *G, const double *C) {
    Nodal m;
    m.n = n;
    m.g.assign(G, G + (size_t)n * n);
    m.c.assign(C, C + (size_t)n * n);
    symmetrise(m.c, n);
    symmetrise(m.g, n);
    m.g_ground.assign(n, 0.0);
    m.c_ground.assign(n, 0.0);
    for (int i = 0; i < n; i++) {
        double sg = 0, sc = 0;
        for (int j = 0; j < n; j++) { sg += m.g[(size_t)i * n + j]; sc += m.c[(size_t)i * n + j]; }
        m.g_ground[i] = sg;
        m.c_ground[i] = sc;
        for (int j = i; j < n; j++) { m.g_total += m.g[(size_t)i * n + j]; m.c_total += m.c[(size_t)i * n + j]; }
    }
    return m;
}

bool valid_names(int32_t n, const char *const *names) {
    if (!names) return false;
    for (int i = 0; i < n; i++)
        if (!names[i]) return false;
    return true;
}

}  // namespace
}  // namespace g2p

// computeYBusFromParam at the first frequency (src/solnoutclass.hpp:1662-1748,
// the dense-matrix build), as saveNetworkParam calls it: from 'Z' the matrix
// itself is taken as Y, from 'Y' its inverse (the reference's two branches);
// G = Re Y and C(i, j) = -1 / (Im Y(i, j) * (2 pi f0)).  'S' is rejected: the
// reference leaves its Y empty there.
extern "C" g2p_status g2p_ybus_from_param(char param, int32_t nports, double freq0, const double *p0, double *G,
                                          double *C) {
    if (nports < 1 || nports > kMaxNetPorts || !p0 || !G || !C || !(param == 'Z' || param == 'Y')) {
        set_last_message(param == 'S' ? "g2p_ybus_from_param: S-parameters have no nodal matrices"
                                      : "g2p_ybus_from_param: invalid argument");
        return param == 'S' ? G2P_ERR_UNSUPPORTED : G2P_ERR_INVALID;
    }
    const int n = nports;
    std::vector<double> y((size_t)2 * n * n);
    if (param == 'Y') {
        G2P_TRY(g2p_convert_param('Y', 'Z', n, 1, nullptr, p0, y.data()));
    } else {
        std::copy(p0, p0 + y.size(), y.begin());
    }
    const double w = 2. * M_PI * freq0;
    for (int t = 0; t < n * n; t++) {
        G[t] = y[2 * t];
        C[t] = -1 / (y[2 * t + 1] * w);
    }
    return G2P_OK;
}

// toXyce (src/solnoutclass.hpp:2094-2225, dense build): a SPICE subcircuit of
// capacitors (inductors where a capacitance is negative), and resistors,
// keeping elements at or above save_thresh times the total.
extern "C" g2p_status g2p_write_xyce(const char *path, const char *design, int32_t nports,
                                     const char *const *port_names, double freq0, const double *G, const double *C,
                                     double save_thresh) {
    if (!path || !design || nports < 1 || !valid_names(nports, port_names) || !G || !C) {
        set_last_message("g2p_write_xyce: invalid argument");
        return G2P_ERR_INVALID;
    }
    try {
        std::ofstream o(path);
        if (!o.is_open()) { set_last_message("g2p_write_xyce: cannot open %s", path); return G2P_ERR_INVALID; }
        const int n = nports;
        const Nodal m = nodal(n, G, C);
        o << "* File: " << path << std::endl;
        o << "* Design: " << design << std::endl;
        o << "* Vendor: DARPA ERI Contributors" << std::endl;
        o << "* Program: Xyce Writer from DARPA ERI" << std::endl;
        o << "* Author: Purdue University" << std::endl;
        o << "* Date: " << timestamp("%d-%m-%Y %H:%M:%S") << std::endl;
        o << std::endl;
        o << ".subckt " << design;
        for (int i = 0; i < n; i++) o << " " << port_names[i];
        o << std::endl;
        const double w2 = std::pow(2. * M_PI * freq0, 2.);
        int ncap = 1, nind = 1, nres = 1;
        for (int i = 0; i < n; i++) {
            for (int j = 0; j < n; j++) {
                if (i == j && std::abs(m.c_ground[i]) >= save_thresh * m.c_total) {
                    const double cng = m.c_ground[i];
                    if (cng > 0.0) o << "C" << ncap++ << " " << port_names[i] << " 0 " << cng << std::endl;
                    else o << "L" << nind++ << " " << port_names[i] << " 0 " << -1.0 / (cng * w2) << std::endl;
                } else if (j > i && std::abs(-m.c[(size_t)i * n + j]) >= save_thresh * m.c_total) {
                    const double cnn = -1.0 * m.c[(size_t)i * n + j];
                    if (cnn > 0.0)
                        o << "C" << ncap++ << " " << port_names[i] << " " << port_names[j] << " " << cnn << std::endl;
                    else
                        o << "L" << nind++ << " " << port_names[i] << " " << port_names[j] << " " << -1.0 / (cnn * w2)
                          << std::endl;
                }
            }
            for (int j = 0; j < n; j++) {
                if (i == j && std::abs(m.g_ground[i]) >= save_thresh * m.g_total)
                    o << "R" << nres++ << " " << port_names[i] << " 0 " << std::abs(1.0 / m.g_ground[i]) << std::endl;
                else if (j > i && std::abs(-1.0 / m.g[(size_t)i * n + j]) >= save_thresh * m.g_total)
                    o << "R" << nres++ << " " << port_names[i] << " " << port_names[j] << " "
                      << std::abs(-1.0 / m.g[(size_t)i * n + j]) << std::endl;
            }
        }
        o << ".ends" << std::endl;
        o.close();
        if (o.fail()) { set_last_message("g2p_write_xyce: write to %s failed", path); return G2P_ERR_INVALID; }
    } catch (const std::exception &e) {
        set_last_message("g2p_write_xyce: %s", e.what());
        return G2P_ERR_INVALID;
    }
    return G2P_OK;
}

// toSPEF + dumpSPEF (src/solnoutclass.hpp:1972-2091, 6008-6030): one net
// "all" connecting every port, with the same capacitor and resistor choices
// as the Xyce writer, in IEEE 1481-1998 syntax.  Ports are referred to
// through the name map (*1, *2, ...); port_dirs holds 'I', 'O' or 'B' per
// port (NULL: all 'B').  The reference prints through the Parser-SPEF
// library, whose exact layout (spacing, blank lines) this writer does not
// reproduce.
extern "C" g2p_status g2p_write_spef(const char *path, const char *design, int32_t nports,
                                     const char *const *port_names, const char *port_dirs, const double *G,
                                     const double *C, double save_thresh) {
    if (!path || !design || nports < 1 || !valid_names(nports, port_names) || !G || !C) {
        set_last_message("g2p_write_spef: invalid argument");
        return G2P_ERR_INVALID;
    }
    try {
        std::ofstream o(path);
        if (!o.is_open()) { set_last_message("g2p_write_spef: cannot open %s", path); return G2P_ERR_INVALID; }
        const int n = nports;
        const Nodal m = nodal(n, G, C);
        auto dir = [&](int i) {
            const char d = port_dirs ? port_dirs[i] : 'B';
            return d == 'O' ? "O" : d == 'I' ? "I" : "B";
        };
        o << "*SPEF \"IEEE 1481-1998\"" << std::endl;
        o << "*DESIGN \"" << design << "\"" << std::endl;
        o << "*DATE \"" << timestamp("%d-%m-%Y %H:%M:%S") << "\"" << std::endl;
        o << "*VENDOR \"DARPA ERI Contributors\"" << std::endl;
        o << "*PROGRAM \"SPEF Writer from DARPA ERI\"" << std::endl;
        o << "*VERSION \"1.0\"" << std::endl;
        o << "*DESIGN_FLOW \"NETLIST_TYPE_VERILOG\"" << std::endl;
        o << "*DIVIDER /" << std::endl;
        o << "*DELIMITER :" << std::endl;
        o << "*BUS_DELIMITER [ ]" << std::endl;
        o << "*T_UNIT 1 S" << std::endl;
        o << "*C_UNIT 1 F" << std::endl;
        o << "*R_UNIT 1 OHM" << std::endl;
        o << "*L_UNIT 1 H" << std::endl << std::endl;
        o << "*NAME_MAP" << std::endl;
        for (int i = 0; i < n; i++) o << "*" << i + 1 << " " << port_names[i] << std::endl;
        o << std::endl << "*PORTS" << std::endl;
        for (int i = 0; i < n; i++) o << "*" << i + 1 << " " << dir(i) << std::endl;
        o << std::endl << "*D_NET all " << m.c_total << std::endl;
        o << "*CONN" << std::endl;
        for (int i = 0; i < n; i++) o << "*P " << port_names[i] << " " << dir(i) << std::endl;
        std::vector<std::string> caps, ress;
        char buf[64];
        auto num = [&](double v) { snprintf(buf, sizeof buf, "%g", v); return std::string(buf); };
        for (int i = 0; i < n; i++) {
            const std::string pi = "*" + std::to_string(i + 1);
            for (int j = 0; j < n; j++) {
                if (i == j && std::abs(m.c_ground[i]) >= save_thresh * m.c_total)
                    caps.push_back(pi + " " + num(m.c_ground[i]));
                else if (j > i && std::abs(-m.c[(size_t)i * n + j]) >= save_thresh * m.c_total)
                    caps.push_back(pi + " *" + std::to_string(j + 1) + " " + num(-m.c[(size_t)i * n + j]));
            }
            for (int j = 0; j < n; j++) {
                if (i == j && std::abs(m.g_ground[i]) >= save_thresh * m.g_total)
                    ress.push_back(pi + " " + num(std::abs(1.0 / m.g_ground[i])));
                else if (j > i && std::abs(-1.0 / m.g[(size_t)i * n + j]) >= save_thresh * m.g_total)
                    ress.push_back(pi + " *" + std::to_string(j + 1) + " " + num(std::abs(-1.0 / m.g[(size_t)i * n + j])));
            }
        }
        o << "*CAP" << std::endl;
        for (size_t k = 0; k < caps.size(); k++) o << k + 1 << " " << caps[k] << std::endl;
        o << "*RES" << std::endl;
        for (size_t k = 0; k < ress.size(); k++) o << k + 1 << " " << ress[k] << std::endl;
        o << "*END" << std::endl;
        o.close();
        if (o.fail()) { set_last_message("g2p_write_spef: write to %s failed", path); return G2P_ERR_INVALID; }
    } catch (const std::exception &e) {
        set_last_message("g2p_write_spef: %s", e.what());
        return G2P_ERR_INVALID;
    }
    return G2P_OK;
}

// ---------------------------------------------------------------------------
// Port termination (Parasitics::terminatePortZ / terminatePortY,
// src/solnoutclass.hpp:1767-1921) and the circuit's Y-parameters
// (computeYParamFromCircuit, :1617-1678).
namespace g2p {
namespace {

// Kron reduction of port k loaded by l[f]: p'_ij = p_ij - p_ik p_kj / (p_kk + l)
// for i, j != k, one thread per output entry of every frequency
__global__ void k_kron(int n, int nfreq, int k, const double *in, const double *load, double *out) {
    const int m = n - 1;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)nfreq * m * m;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = t / ((int64_t)m * m);
        const int r = (int)(t % ((int64_t)m * m));
        const int i = r / m + (r / m >= k ? 1 : 0), j = r % m + (r % m >= k ? 1 : 0);
        const double *p = in + 2 * f * n * n;
        const Cx pij = {p[2 * (i * n + j)], p[2 * (i * n + j) + 1]};
        const Cx pik = {p[2 * (i * n + k)], p[2 * (i * n + k) + 1]};
        const Cx pkj = {p[2 * (k * n + j)], p[2 * (k * n + j) + 1]};
        const Cx den = cadd({p[2 * (k * n + k)], p[2 * (k * n + k) + 1]}, {load[2 * f], load[2 * f + 1]});
        const Cx v = csub(pij, cdiv(cmul(pik, pkj), den));
        out[2 * t] = v.re;
        out[2 * t + 1] = v.im;
    }
}

__global__ void k_y_circuit(int n, int nfreq, const double *freqs, const double *G, const double *C, double *out) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)nfreq * n * n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = t / ((int64_t)n * n);
        const int e = (int)(t % ((int64_t)n * n));
        out[2 * t] = G[e];
        out[2 * t + 1] = 2. * 3.14159265358979323846 * freqs[f] * C[e];
    }
}

}  // namespace
}  // namespace g2p

extern "C" g2p_status g2p_terminate_port(char param, int32_t nports, int32_t nfreq, const double *freqs, int32_t port,
                                         int32_t nload, const double *load, const double *in, double *out) {
    if ((param != 'Z' && param != 'Y') || nports < 2 || nfreq < 1 || port < 0 || port >= nports || !freqs || !load ||
        !in || !out) {
        set_last_message("g2p_terminate_port: Z or Y parameters, 2 or more ports, a port index in range");
        return G2P_ERR_INVALID;
    }
    if (nload != 1 && nfreq == 1) {
        set_last_message("g2p_terminate_port: %d load values for one frequency", nload);
        return G2P_ERR_INVALID;
    }
    // the load at the first frequency, its imaginary part scaled with
    // frequency (the reference's rule whenever the sweep has more than one
    // point or one load value is given)
    std::vector<double> f(nfreq), l(2 * (size_t)nfreq);
    double l0[2];
    G2P_CUDA(cudaMemcpy(f.data(), freqs, sizeof(double) * nfreq, cudaMemcpyDefault));
    G2P_CUDA(cudaMemcpy(l0, load, sizeof(double) * 2, cudaMemcpyDefault));
    for (int q = 0; q < nfreq; q++) {
        l[2 * q] = l0[0];
        l[2 * q + 1] = l0[1] * f[q] / f[0];
    }
    const int64_t nin = 2LL * nfreq * nports * nports, nout = 2LL * nfreq * (nports - 1) * (nports - 1);
    cudaStream_t s;
    G2P_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    double *d_in = nullptr, *d_out = nullptr, *d_l = nullptr;
    auto run = [&]() -> g2p_status {
        G2P_TRY(dalloc(&d_in, nin, s));
        G2P_TRY(dalloc(&d_out, nout, s));
        G2P_TRY(dalloc(&d_l, 2LL * nfreq, s));
        G2P_CUDA(cudaMemcpyAsync(d_in, in, sizeof(double) * nin, cudaMemcpyDefault, s));
        G2P_CUDA(cudaMemcpyAsync(d_l, l.data(), sizeof(double) * 2 * nfreq, cudaMemcpyHostToDevice, s));
        (kbegin("k_kron", s), k_kron<<<grid_for(nout / 2), kThreads, 0, s>>>(nports, nfreq, port, d_in, d_l, d_out), kend(s));
        G2P_CUDA(cudaMemcpyAsync(out, d_out, sizeof(double) * nout, cudaMemcpyDefault, s));
        G2P_CUDA(cudaStreamSynchronize(s));
        return G2P_OK;
    };
    g2p_status st = run();
    dfree(d_in, s); dfree(d_out, s); dfree(d_l, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return st;
}

extern "C" g2p_status g2p_y_from_circuit(int32_t nports, int32_t nfreq, const double *freqs, const double *G,
                                         const double *C, double *out) {
    if (nports < 1 || nfreq < 1 || !freqs || !G || !C || !out) {
        set_last_message("g2p_y_from_circuit: bad arguments");
        return G2P_ERR_INVALID;
    }
    const int64_t nn = (int64_t)nports * nports, nout = 2LL * nfreq * nn;
    cudaStream_t s;
    G2P_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    double *d_f = nullptr, *d_g = nullptr, *d_c = nullptr, *d_o = nullptr;
    auto run = [&]() -> g2p_status {
        G2P_TRY(dalloc(&d_f, nfreq, s));
        G2P_TRY(dalloc(&d_g, nn, s));
        G2P_TRY(dalloc(&d_c, nn, s));
        G2P_TRY(dalloc(&d_o, nout, s));
        G2P_CUDA(cudaMemcpyAsync(d_f, freqs, sizeof(double) * nfreq, cudaMemcpyDefault, s));
        G2P_CUDA(cudaMemcpyAsync(d_g, G, sizeof(double) * nn, cudaMemcpyDefault, s));
        G2P_CUDA(cudaMemcpyAsync(d_c, C, sizeof(double) * nn, cudaMemcpyDefault, s));
        (kbegin("k_y_circuit", s), k_y_circuit<<<grid_for(nout / 2), kThreads, 0, s>>>(nports, nfreq, d_f, d_g, d_c, d_o), kend(s));
        G2P_CUDA(cudaMemcpyAsync(out, d_o, sizeof(double) * nout, cudaMemcpyDefault, s));
        G2P_CUDA(cudaStreamSynchronize(s));
        return G2P_OK;
    };
    g2p_status st = run();
    dfree(d_f, s); dfree(d_g, s); dfree(d_c, s); dfree(d_o, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return st;
}
