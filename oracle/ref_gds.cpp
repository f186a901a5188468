/* Runs the reference's own GDSII database (AsciiDataBase) and saveToMesh
 * (limboint.hpp), compiled unmodified with the project's stream-reader
 * stand-in, on one GDSII file, and prints the conductor polygons that
 * saveToMesh leaves in fdtdMesh::conductorIn: one line per polygon,
 * "P layer nvert x0 y0 x1 y1 ..." (metres, %.17g); other lines are the
 * reference's own messages.  The top cell is the last
 * cell of the file, as the reference's command-line driver takes it.
 * With --grid <settings>, it then fills the remaining fdtdMesh members the
 * way the reference's convertToFDTDMesh does (solnoutclass.hpp:5894-5984):
 * limits, the layer stack, each polygon's z range from the stack layer with
 * its GDSII number, the port sides; runs the reference's meshAndMark
 * (mesh.cpp:5) and prints its grid lines and per-layer constants as lines
 * "X x0 x1 ...", "Y ...", "Z ...", "E eps ...", "S sigma ...".  The settings
 * file holds: xlim1 xlim2 ylim1 ylim2 zlim1 zlim2 / nstack, then per layer
 * "z_begin z_end eps sigma gdsii_number" / nport, then per port side
 * "x1 y1 z1 x2 y2 z2 direction" (one side per port), all lengths in metres.
 * With --mark <settings> <dump_dir> it does the same with ports of several
 * sides each (the settings' port section is then: nport, and per port its
 * side count followed by one "x1 y1 z1 x2 y2 z2 direction" line per side),
 * runs meshAndMark (grid, findInsideCond marking, conductor numbering,
 * findPortNode, markPort, boundary sets, setMapEdge, markEdge recolouring)
 * and portSet (mesh.cpp:1196), and writes into dump_dir: mark_node.i64,
 * mark_edge.i64, map_edge.i64, the grid (xn/yn/zn.f64) and per-layer constants
 * (stack_epsn/stack_sign.f64), mark_port.i32 per
 * conductor, per port side its edges (side_edges.i64 with
 * side_edge_ptr.i64), area and direction, the side coordinates after
 * findPortNode (side_coords.f64), and meta.txt (nx ny nz numCdt bden status).
 * TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.sh into oracle/_ref/.
 * usage: ref_gds <file.gds> [--grid settings | --mark settings dump_dir] [ignored GDSII layer ...] */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <unordered_set>
#include "limboint.hpp"

int meshAndMark(fdtdMesh *sys, unordered_map<double, int> &xi, unordered_map<double, int> &yi,
                unordered_map<double, int> &zi, unordered_set<double> *portCoorx, unordered_set<double> *portCoory);

int portSet(fdtdMesh *sys, unordered_map<double, int> xi, unordered_map<double, int> yi, unordered_map<double, int> zi);

template <class T> static void dump(const std::string &dir, const char *name, const T *p, size_t n) {
    FILE *f = fopen((dir + "/" + name).c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s/%s\n", dir.c_str(), name); exit(3); }
    if (n) fwrite(p, sizeof(T), n, f);
    fclose(f);
}

int main(int argc, char **argv) {
    if (argc < 2) { fprintf(stderr, "usage: ref_gds <file.gds> [ignored layer ...]\n"); return 2; }
    AsciiDataBase adb;
    adb.setFileName(argv[1]);
    GdsParser::GdsReader rd(adb);
    if (!rd(argv[1])) { fprintf(stderr, "cannot read %s\n", argv[1]); return 3; }
    std::vector<int> ignore;
    const char *grid = nullptr, *dumpdir = nullptr;
    for (int i = 2; i < argc; i++) {
        if (!strcmp(argv[i], "--grid") && i + 1 < argc) grid = argv[++i];
        else if (!strcmp(argv[i], "--mark") && i + 2 < argc) { grid = argv[++i]; dumpdir = argv[++i]; }
        else ignore.push_back(atoi(argv[i]));
    }
    fdtdMesh sys;
    const std::string top = adb.getCell(adb.getNumCell() - 1).getCellName();
    adb.saveToMesh(top, {0., 0.}, strans(), &sys, ignore);
    for (size_t i = 0; i < sys.conductorIn.size(); i++) {
        const fdtdOneCondct &c = sys.conductorIn[i];
        printf("P %d %d", (int)c.layer, (int)c.numVert);
        for (int v = 0; v < c.numVert; v++) printf(" %.17g %.17g", c.x[v], c.y[v]);
        printf("\n");
    }
    if (!grid) return 0;
    std::ifstream in(grid);
    double lim[6];
    for (double &v : lim) in >> v;
    sys.xlim1 = lim[0]; sys.xlim2 = lim[1]; sys.ylim1 = lim[2]; sys.ylim2 = lim[3]; sys.zlim1 = lim[4]; sys.zlim2 = lim[5];
    int ns = 0;
    in >> ns;
    sys.numStack = ns;
    std::vector<int> gds(ns);
    for (int k = 0; k < ns; k++) {
        double b, e, eps, sig;
        in >> b >> e >> eps >> sig >> gds[k];
        sys.stackBegCoor.push_back(b); sys.stackEndCoor.push_back(e);
        sys.stackEps.push_back(eps); sys.stackSig.push_back(sig);
        sys.stackName.push_back(std::to_string(gds[k]));
    }
    sys.numCdtRow = (int)sys.conductorIn.size();
    sys.stackCdtMark = (double *)calloc(ns > 0 ? ns : 1, sizeof(double));
    for (int i = 0; i < sys.numCdtRow; i++)
        for (int k = 0; k < ns; k++)
            if (sys.conductorIn[i].layer == gds[k]) {
                sys.conductorIn[i].zmin = sys.stackBegCoor[k];
                sys.conductorIn[i].zmax = sys.stackEndCoor[k];
                sys.stackCdtMark[k] = 1;
            }
    int np = 0;
    in >> np;
    sys.numPorts = np;
    unordered_set<double> pcx, pcy;
    for (int p = 0; p < np; p++) {
        int mult = 1;
        if (dumpdir) in >> mult;
        sys.portCoor.emplace_back(fdtdPort());
        fdtdPort &pc = sys.portCoor.back();
        for (int k = 0; k < mult; k++) {
            double c[6];
            int dir;
            for (double &v : c) in >> v;
            in >> dir;
            pc.x1.push_back(c[0]); pc.y1.push_back(c[1]); pc.z1.push_back(c[2]);
            pc.x2.push_back(c[3]); pc.y2.push_back(c[4]); pc.z2.push_back(c[5]);
            pc.portDirection.push_back(dir);
            /* convertToFDTDMesh (solnoutclass.hpp:5966-5977) records the first
               side's coordinates only */
            if (k == 0 && c[0] == c[3]) pcx.insert(c[0]);
            if (k == 0 && c[1] == c[4]) pcy.insert(c[1]);
        }
        pc.multiplicity = mult;
    }
    unordered_map<double, int> xi, yi, zi;
    const int st = meshAndMark(&sys, xi, yi, zi, &pcx, &pcy);
    auto line = [](const char *tag, const double *v, long n) {
        printf("%s", tag);
        for (long i = 0; i < n; i++) printf(" %.17g", v[i]);
        printf("\n");
    };
    line("X", sys.xn, sys.nx);
    line("Y", sys.yn, sys.ny);
    line("Z", sys.zn, sys.nz);
    line("E", sys.stackEpsn.data(), (long)sys.stackEpsn.size());
    line("S", sys.stackSign.data(), (long)sys.stackSign.size());
    printf("STATUS %d\n", st);
    if (!dumpdir) return 0;
    const std::string dd = dumpdir;
    int st2 = -1;
    if (st == 0) st2 = portSet(&sys, xi, yi, zi);
    std::ofstream meta(dd + "/meta.txt");
    meta << sys.nx << " " << sys.ny << " " << sys.nz << " " << (st == 0 ? (long long)sys.numCdt : 0LL) << " "
         << (long long)sys.bden << " " << st << " " << st2 << "\n";
    meta.close();
    dump(dd, "xn.f64", sys.xn, sys.nx);
    dump(dd, "yn.f64", sys.yn, sys.ny);
    dump(dd, "zn.f64", sys.zn, sys.nz);
    dump(dd, "stack_epsn.f64", sys.stackEpsn.data(), sys.stackEpsn.size());
    dump(dd, "stack_sign.f64", sys.stackSign.data(), sys.stackSign.size());
    if (st != 0) return 0;
    dump(dd, "mark_node.i64", (const int64_t *)sys.markNode, (size_t)sys.N_node);
    dump(dd, "mark_edge.i64", (const int64_t *)sys.markEdge, (size_t)sys.N_edge);
    dump(dd, "map_edge.i64", (const int64_t *)sys.mapEdge, (size_t)sys.N_edge);
    std::vector<int32_t> mp((size_t)sys.numCdt);
    for (long long c = 0; c < (long long)sys.numCdt; c++) mp[(size_t)c] = sys.conductor[c].markPort;
    dump(dd, "mark_port.i32", mp.data(), mp.size());
    if (st2 != 0) return 0;
    std::vector<int64_t> eptr(1, 0), edges;
    std::vector<double> area, coords;
    std::vector<int32_t> dirs;
    for (int p = 0; p < np; p++) {
        const fdtdPort &pc = sys.portCoor[p];
        for (int k = 0; k < pc.multiplicity; k++) {
            for (auto e : pc.portEdge[k]) edges.push_back((int64_t)e);
            eptr.push_back((int64_t)edges.size());
            area.push_back(pc.portArea[k]);
            dirs.push_back(pc.portDirection[k]);
            for (double v : {pc.x1[k], pc.y1[k], pc.z1[k], pc.x2[k], pc.y2[k], pc.z2[k]}) coords.push_back(v);
        }
    }
    dump(dd, "side_edge_ptr.i64", eptr.data(), eptr.size());
    dump(dd, "side_edges.i64", edges.data(), edges.size());
    dump(dd, "side_area.f64", area.data(), area.size());
    dump(dd, "side_dir.i32", dirs.data(), dirs.size());
    dump(dd, "side_coords.f64", coords.data(), coords.size());
    return 0;
}
