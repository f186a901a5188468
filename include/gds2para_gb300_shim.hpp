/* Reference-signature shim for gds2Para's V0 path (C++17, header only).
 *
 * generateStiff, hypreSolve and paraGenerator with the reference's argument
 * lists and effects, forwarded to the C ABI of gds2para_gb300.h:
 *
 *   generateStiff(fdtdMesh *)                    src/generateStiff.cpp:6
 *   hypreSolve(fdtdMesh *, myint *ARowId, ...)   src/hypreSolve.cpp:9, src/hypreSolver.h:14
 *   paraGenerator(fdtdMesh *, xi, yi, zi)        src/matrixCon.cpp:11
 *
 * The functions are templates over the mesh type.  They read and write only
 * these fdtdMesh members (src/fdtd.hpp:182-356): N_cell_x/y/z, xn/yn/zn,
 * stackEpsn, stackSign, markNode, markEdge, numCdt, conductor[].markPort
 * (and conductor[].node, freed as the reference frees it), numPorts,
 * portCoor[].multiplicity/portEdge/portArea/portDirection,
 * freqStart/freqEnd/freqUnit/nfreq/freqScale, SRowId/SColId/Sval/leng_S,
 * x and Y.  gds2Para instantiates them with its own fdtdMesh in one
 * translation unit (see the three forwarding definitions at the end of this
 * comment); tests instantiate them with a struct that has the same members.
 *
 *   #include "fdtd.hpp"
 *   #include "gds2para_gb300_shim.hpp"
 *   int generateStiff(fdtdMesh *sys) { return g2p_shim::generateStiff(sys); }
 *   int hypreSolve(fdtdMesh *sys, myint *r, myint *c, double *v, myint nnz, double *b, myint n, double *x) {
 *       return g2p_shim::hypreSolve(sys, r, c, v, nnz, b, n, x);
 *   }
 *   int paraGenerator(fdtdMesh *sys, unordered_map<double, int> xi, unordered_map<double, int> yi,
 *                     unordered_map<double, int> zi) {
 *       return g2p_shim::paraGenerator(sys, xi, yi, zi);
 *   }
 *
 * Behaviour kept from the reference: generateStiff mallocs SRowId/SColId/
 * Sval (int64 COO, freed by ~fdtdMesh); hypreSolve reads a row-sorted 0-based
 * COO and overwrites the caller's solution with hypreSolve's settings
 * (FlexGMRES KDim 10, 100 iterations, rtol 1e-4); paraGenerator assigns
 * sys->x (nfreq * P * P complex, frequencies after the first stored
 * transposed as print_z_V0 does), callocs sys->Y, and frees markNode,
 * conductor (with each conductor's node list) and xn/yn/zn and clears
 * stackEpsn, as src/matrixCon.cpp:182-187,893-896 do.
 * Differences: a failure returns the nonzero g2p_status and prints
 * g2p_last_error() on stderr (the reference's hypreSolve returns 0 whatever
 * happens), and the whole V0 solve runs on the GPU, not through hypreSolve.
 *
 * generateStiff keeps its device mesh for the paraGenerator call that
 * follows on the same fdtdMesh (the reference's order, TestMain.cpp:343,370),
 * so S is built once.  One mesh at a time per process. */
#ifndef GDS2PARA_GB300_SHIM_HPP
#define GDS2PARA_GB300_SHIM_HPP

#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <type_traits>
#include <vector>

#include "gds2para_gb300.h"

namespace g2p_shim {

/* Solver settings of paraGenerator's V0 solves; change before the call. */
struct Settings {
    int32_t precision = G2P_PREC_MIXED;   /* FP32 AMG-FGMRES inside FP64 refinement */
    double rtol = 1e-8;
    int32_t batch = 1;                    /* all ports as one block of right-hand sides */
    int32_t autotune = 0;
    bool reference_frees = true;          /* free markNode, conductor, xn/yn/zn as the reference does */
};

inline Settings &settings() {
    static Settings s;
    return s;
}

/* Host staging of the fdtdMesh fields the descriptor points at, and the
 * device mesh built from them. */
struct Staging {
    const void *owner = nullptr;
    std::vector<int32_t> mark_port, side_ptr, side_dir;
    std::vector<uint8_t> cdt_return;
    std::vector<int64_t> edge_ptr, edges;
    std::vector<double> area;
    g2p_mesh *h = nullptr;
    ~Staging() {
        if (h) g2p_mesh_destroy(h);
    }
};

inline Staging *&current() {
    static Staging *g = nullptr;
    return g;
}

inline int report(g2p_status s, const char *what) {
    if (s != G2P_OK) std::fprintf(stderr, "gds2para_gb300: %s: %s\n", what, g2p_last_error());
    return (int)s;
}

/* g2p_mesh_create from the fdtdMesh that meshAndMark, matrixConstruction and
 * portSet leave (src/mesh.cpp:5-1594).  cdt_return[c] = 1 for the
 * conductors mesh.cpp:943-953 hands to findBoundNodeEdge: the ports' return
 * conductors (markPort == -1). */
template <class Mesh>
g2p_status open_mesh(Mesh *sys, Staging &g) {
    static_assert(sizeof(*sys->markNode) == sizeof(int64_t), "myint must be 64 bits");
    for (int64_t c = 0; c < (int64_t)sys->numCdt; c++) {
        g.mark_port.push_back(sys->conductor[c].markPort);
        g.cdt_return.push_back(sys->conductor[c].markPort == -1);
    }
    g.side_ptr.push_back(0);
    g.edge_ptr.push_back(0);
    for (int p = 0; p < sys->numPorts; p++) {
        const auto &pc = sys->portCoor[p];
        for (int s = 0; s < pc.multiplicity; s++) {
            for (auto e : pc.portEdge[s]) g.edges.push_back((int64_t)e);
            g.edge_ptr.push_back((int64_t)g.edges.size());
            g.area.push_back(pc.portArea[s]);
            g.side_dir.push_back(pc.portDirection[s]);
        }
        g.side_ptr.push_back((int32_t)g.area.size());
    }
    g2p_mesh_desc d = {};
    d.nx = (int64_t)sys->N_cell_x + 1;
    d.ny = (int64_t)sys->N_cell_y + 1;
    d.nz = (int64_t)sys->N_cell_z + 1;
    d.xn = sys->xn;
    d.yn = sys->yn;
    d.zn = sys->zn;
    d.stack_epsn = sys->stackEpsn.data();
    d.stack_sign = sys->stackSign.data();
    /* myint is long long; the ABI's int64_t may be long: same width and layout */
    d.mark_node = reinterpret_cast<const int64_t *>(sys->markNode);
    d.mark_edge = reinterpret_cast<const int64_t *>(sys->markEdge);
    d.num_cdt = (int64_t)sys->numCdt;
    d.mark_port = g.mark_port.data();
    d.cdt_return = g.cdt_return.data();
    d.num_ports = sys->numPorts;
    d.port_side_ptr = g.side_ptr.data();
    d.side_edge_ptr = g.edge_ptr.data();
    d.side_edges = g.edges.data();
    d.side_area = g.area.data();
    d.side_dir = g.side_dir.data();
    d.freq_start = sys->freqStart;
    d.freq_end = sys->freqEnd;
    d.freq_unit = sys->freqUnit;
    d.nfreq = sys->nfreq;
    d.freq_scale = sys->freqScale;
    return g2p_mesh_create(&d, &g.h);   /* copies everything it needs */
}

/* The device mesh of `sys`, built on first use. */
template <class Mesh>
g2p_status mesh_for(Mesh *sys, Staging **out) {
    Staging *&g = current();
    if (g && g->owner != (const void *)sys) {
        delete g;
        g = nullptr;
    }
    if (!g) {
        g = new Staging();
        g->owner = sys;
        g2p_status s = open_mesh(sys, *g);
        if (s != G2P_OK) {
            delete g;
            g = nullptr;
            return s;
        }
    }
    *out = g;
    return G2P_OK;
}

inline void close_mesh() {
    delete current();
    current() = nullptr;
}

/* generateStiff (src/generateStiff.cpp:6-565): S on the device, exported to
 * the reference's SRowId/SColId/Sval COO (malloc'd; ~fdtdMesh frees it). */
template <class Mesh>
int generateStiff(Mesh *sys) {
    Staging *g = nullptr;
    g2p_status s = mesh_for(sys, &g);
    if (s != G2P_OK) return report(s, "generateStiff: mesh");
    int64_t leng = 0;
    if ((s = g2p_generate_stiff(g->h, &leng)) != G2P_OK) return report(s, "generateStiff");
    using Int = typename std::remove_pointer<decltype(sys->SRowId)>::type;
    sys->leng_S = (Int)leng;
    const size_t n = (size_t)(leng > 0 ? leng : 1);
    sys->SRowId = (Int *)std::malloc(sizeof(Int) * n);
    sys->SColId = (Int *)std::malloc(sizeof(Int) * n);
    sys->Sval = (double *)std::malloc(sizeof(double) * n);
    if (!sys->SRowId || !sys->SColId || !sys->Sval) return report(G2P_ERR_NOMEM, "generateStiff: host COO");
    s = g2p_export_stiff(g->h, reinterpret_cast<int64_t *>(sys->SRowId), reinterpret_cast<int64_t *>(sys->SColId),
                         sys->Sval);
    return report(s, "generateStiff: export");
}

/* hypreSolve (src/hypreSolve.cpp:9-283) with the reference's settings. */
template <class Mesh, class Int>
int hypreSolve(Mesh *, Int *ARowId, Int *AColId, double *Aval, Int leng_A, double *bin, Int leng_v0,
               double *solution) {
    static_assert(sizeof(Int) == sizeof(int64_t), "myint must be 64 bits");
    g2p_status s = g2p_hypre_solve(reinterpret_cast<const int64_t *>(ARowId), reinterpret_cast<const int64_t *>(AColId),
                                   Aval, (int64_t)leng_A, bin, (int64_t)leng_v0, solution);
    return report(s, "hypreSolve");
}

/* paraGenerator's V0 path (src/matrixCon.cpp:11-907 with SKIP_VH): Z in
 * sys->x.  The grid-line maps are unused (the reference passes them by
 * value and uses them only in the compiled-out Vh code). */
template <class Mesh, class Map>
int paraGenerator(Mesh *sys, const Map &, const Map &, const Map &) {
    Staging *g = nullptr;
    g2p_status s = mesh_for(sys, &g);
    if (s != G2P_OK) return report(s, "paraGenerator: mesh");
    const Settings &cfg = settings();
    g2p_solver_params p;
    g2p_default_params(&p, 0);
    p.precision = cfg.precision;
    p.rtol = cfg.rtol;
    p.batch = cfg.batch;
    p.autotune = cfg.autotune;
    const size_t nz = (size_t)sys->nfreq * sys->numPorts * sys->numPorts;
    using C = typename std::remove_pointer<decltype(sys->Y)>::type;
    sys->Y = (C *)std::calloc(nz > 0 ? nz : 1, sizeof(C));
    sys->x.assign(nz, std::complex<double>(0., 0.));
    g2p_extract_stats st;
    s = g2p_para_generator(g->h, &p, reinterpret_cast<double *>(sys->x.data()), &st);
    close_mesh();
    if (s != G2P_OK) return report(s, "paraGenerator");
    if (cfg.reference_frees) {
        std::free(sys->markNode);
        sys->markNode = nullptr;
        for (int64_t c = 0; c < (int64_t)sys->numCdt; c++) {
            std::free(sys->conductor[c].node);
            sys->conductor[c].node = nullptr;
        }
        std::free(sys->conductor);
        sys->conductor = nullptr;
        std::free(sys->xn);
        sys->xn = nullptr;
        std::free(sys->yn);
        sys->yn = nullptr;
        std::free(sys->zn);
        sys->zn = nullptr;
        sys->stackEpsn.clear();
    }
    return 0;
}

}  // namespace g2p_shim

#endif
