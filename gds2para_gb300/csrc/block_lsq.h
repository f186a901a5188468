// Host least squares of block FGMRES (block_krylov.cu): plain C++, no CUDA,
// so the CPU tests can compile it on its own.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <vector>

namespace g2p {

// Givens rotations of the block upper-Hessenberg least-squares problem
// min || E1 B0 - Hbar Y ||_F.  A dead index (a basis column that the
// Cholesky QR zeroed as dependent) has a zero row and a zero column in Hbar
// and a zero row in the right-hand side, so it is left out: the rotations
// run over the live rows only, each live column eliminating everything below
// its pivot, and its unknowns stay zero.
struct BlockLSQ {
    struct Rot {
        int r0;
        double c, s;
    };
    int K = 0;
    std::vector<int> live;                 // raw row (basis column) of each live row
    std::vector<char> is_live;             // by raw index
    std::vector<std::vector<double>> col;  // rotated live columns (over live rows)
    std::vector<int> craw;                 // raw index of each live column
    std::vector<Rot> rots;
    std::vector<double> g;                 // live rows x K right-hand sides
    void reset(int k, int m, const double *B0) {
        K = k;
        live.clear(); col.clear(); craw.clear(); rots.clear(); g.clear();
        is_live.assign((size_t)(m + 2) * K, 0);
        for (int p = 0; p < K; p++)
            if (B0[p * K + p] != 0.0) {
                live.push_back(p);
                is_live[p] = 1;
                g.insert(g.end(), B0 + p * K, B0 + p * K + K);
            }
    }
    void rotate_g(const Rot &r) {
        double *g0 = &g[(size_t)r.r0 * K], *g1 = g0 + K;
        for (int q = 0; q < K; q++) {
            const double x0 = g0[q], x1 = g1[q];
            g0[q] = r.c * x0 + r.s * x1;
            g1[q] = -r.s * x0 + r.c * x1;
        }
    }
    // block column j from hcol ((j+2)K rows x K, row-major; rows (j+1)K..
    // hold R, whose zero pivots mark the next block's dead columns); returns
    // each right-hand side's residual norm in res[K]
    void add_block(int j, const double *hcol, double *res) {
        const double *R = hcol + (size_t)(j + 1) * K * K;
        for (int p = 0; p < K; p++)
            if (R[p * K + p] != 0.0) {
                live.push_back((j + 1) * K + p);
                is_live[(size_t)(j + 1) * K + p] = 1;
                g.insert(g.end(), K, 0.0);
            }
        const int nr = (int)live.size(), rows = (j + 2) * K;
        for (int q = 0; q < K; q++) {
            const int c = j * K + q;
            if (!is_live[c]) continue;
            std::vector<double> h(nr);
            for (int i = 0; i < nr; i++) h[i] = live[i] < rows ? hcol[(size_t)live[i] * K + q] : 0.0;
            for (const Rot &r : rots) {
                const double a = h[r.r0], b = h[r.r0 + 1];
                h[r.r0] = r.c * a + r.s * b;
                h[r.r0 + 1] = -r.s * a + r.c * b;
            }
            const int piv = (int)col.size();
            for (int i = nr - 1; i > piv; i--) {
                const double a = h[i - 1], b = h[i];
                if (b == 0.0) continue;
                const double rr = std::hypot(a, b);
                const Rot r{i - 1, a / rr, b / rr};
                h[i - 1] = rr;
                h[i] = 0.0;
                rots.push_back(r);
                rotate_g(r);
            }
            col.push_back(std::move(h));
            craw.push_back(c);
        }
        const int nl = (int)col.size();
        for (int q = 0; q < K; q++) {
            double s = 0;
            for (int i = nl; i < nr; i++) s += g[(size_t)i * K + q] * g[(size_t)i * K + q];
            res[q] = std::sqrt(s);
        }
    }
    // Y (nc x K raw rows, row-major) from the triangular live part; a pivot
    // that is zero relative to the largest leaves its unknown at zero
    void solve(int nc, double *Y) const {
        const int nl = (int)col.size();
        double hmax = 0;
        for (int i = 0; i < nl; i++) hmax = std::max(hmax, std::fabs(col[i][i]));
        std::vector<double> y((size_t)nl * K, 0.0);
        for (int i = nl - 1; i >= 0; i--) {
            const double d = col[i][i];
            const bool ok = std::fabs(d) > 1e-300 + 1e-15 * hmax;
            for (int q = 0; q < K; q++) {
                double v = g[(size_t)i * K + q];
                for (int i2 = i + 1; i2 < nl; i2++) v -= col[i2][i] * y[(size_t)i2 * K + q];
                y[(size_t)i * K + q] = ok ? v / d : 0.0;
            }
        }
        std::fill(Y, Y + (size_t)nc * K, 0.0);
        for (int i = 0; i < nl; i++)
            if (craw[i] < nc) std::copy(&y[(size_t)i * K], &y[(size_t)i * K] + K, Y + (size_t)craw[i] * K);
    }
};

}  // namespace g2p
