/* Runs the reference's own output stage and .sim_input reader
 * (src/solnoutclass.hpp, compiled unmodified against the project's Eigen
 * and Parser-SPEF stand-ins in oracle/ref_shims/) for the fixtures of
 * tests/golden/make_network_golden.py.
 *
 *   ref_network network <in.txt> <out_dir> <design>
 *       in.txt: "nports nfreq", the frequencies (Hz), per port
 *       "name direction z_source", then nfreq*P*P complex Z values
 *       ("re im", sys->x's order).  As TestMain.cpp:385-440 does:
 *       Parasitics::saveNetworkParam('Z', ...) (which runs
 *       computeYBusFromParam(0)), then the writers dumpTouchstone, dumpXyce
 *       and dumpSPEF on the Z data, convertParam('S') and dumpCITI and
 *       dumpTouchstone on the S data; and convertParam for every pair of
 *       kinds.  Writes G.txt, C.txt (nodal matrices), Z_to_{Y,S}.txt,
 *       S_to_{Y,Z}.txt, Y_to_{S,Z}.txt (one "re im" pair per entry, %.17g)
 *       and the files z.ts, z.cir, z.spef, s.citi, s.ts.
 *   ref_network simin <file.sim_input> <out.txt>
 *       SolverDataBase::readSimInput and convertToFDTDMesh: the fdtdMesh
 *       limits, frequency fields, stack (with the valid layers' GDSII
 *       numbers) and port sides with their directions, one value per token.
 * TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.sh into oracle/_ref/. */
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <unordered_set>
#include <vector>

#include "solnoutclass.hpp"

static void dump_mats(const std::string &path, const std::vector<cdMat> &m) {
    FILE *f = fopen(path.c_str(), "w");
    for (const auto &a : m)
        for (long i = 0; i < a.rows(); i++)
            for (long j = 0; j < a.cols(); j++) fprintf(f, "%.17g %.17g\n", a(i, j).real(), a(i, j).imag());
    fclose(f);
}

static void dump_real(const std::string &path, const dMat &m) {
    FILE *f = fopen(path.c_str(), "w");
    for (long i = 0; i < m.rows(); i++)
        for (long j = 0; j < m.cols(); j++) fprintf(f, "%.17g\n", m(i, j));
    fclose(f);
}

static int network(const char *in, const std::string &out, const std::string &design) {
    std::ifstream f(in);
    size_t np = 0, nf = 0;
    f >> np >> nf;
    std::vector<double> freqs(nf);
    for (auto &v : freqs) f >> v;
    std::vector<Port> ports;
    for (size_t p = 0; p < np; p++) {
        std::string name;
        char dir;
        double zs;
        f >> name >> dir >> zs;
        ports.emplace_back(Port(name, dir, zs, 1, {0., 0., 0., 0., 0., 0.}, -1));
    }
    std::vector<complex<double>> x(nf * np * np);
    for (auto &v : x) {
        double re, im;
        f >> re >> im;
        v = complex<double>(re, im);
    }
    Parasitics para(ports, dMat(np, np), dMat(np, np), freqs);
    para.saveNetworkParam('Z', freqs, x);
    dump_real(out + "/G.txt", para.getGMatrix());
    dump_real(out + "/C.txt", para.getCMatrix());
    SolverDataBase sdb;
    sdb.setDesignName(design);
    sdb.setParasitics(para);
    sdb.setOutTouchstone(out + "/z.ts");
    sdb.setOutXyce(out + "/z.cir");
    sdb.setOutSPEF(out + "/z.spef");
    if (!sdb.dumpTouchstone() || !sdb.dumpXyce() || !sdb.dumpSPEF()) return 3;
    const char kinds[3] = {'Z', 'Y', 'S'};
    for (char from : kinds)
        for (char to : kinds) {
            if (from == to) continue;
            Parasitics q = para;
            if (from != 'Z') q.convertParam(from);
            q.convertParam(to);
            dump_mats(out + "/" + from + "_to_" + to + ".txt", q.getParamMatrix());
            if (from == 'Z' && to == 'S') {
                SolverDataBase s2;
                s2.setDesignName(design);
                s2.setParasitics(q);
                s2.setOutCITI(out + "/s.citi");
                s2.setOutTouchstone(out + "/s.ts");
                if (!s2.dumpCITI() || !s2.dumpTouchstone()) return 4;
            }
        }
    return 0;
}

static int simin(const char *path, const char *out) {
    SolverDataBase sdb;
    if (!sdb.readSimInput(path)) return 2;
    fdtdMesh sys;
    unordered_set<double> pcx, pcy;
    sdb.convertToFDTDMesh(&sys, 0, &pcx, &pcy);
    FILE *f = fopen(out, "w");
    fprintf(f, "lim %.17g %.17g %.17g %.17g %.17g %.17g\n", sys.xlim1, sys.xlim2, sys.ylim1, sys.ylim2, sys.zlim1,
            sys.zlim2);
    fprintf(f, "units %.17g %.17g %.17g %.17g\n", sys.lengthUnit, sys.freqUnit, sys.freqStart, sys.freqEnd);
    fprintf(f, "freq %d %d\n", (int)sys.nfreq, (int)sys.freqScale);
    const vector<Layer> valid = sdb.getValidLayers();
    for (size_t k = 0; k < (size_t)sys.numStack; k++)
        fprintf(f, "layer %.17g %.17g %.17g %.17g %d\n", sys.stackBegCoor[k], sys.stackEndCoor[k], sys.stackEps[k],
                sys.stackSig[k], valid[k].getGDSIINum());
    for (int p = 0; p < sys.numPorts; p++) {
        const fdtdPort &pc = sys.portCoor[p];
        for (int k = 0; k < pc.multiplicity; k++)
            fprintf(f, "side %d %.17g %.17g %.17g %.17g %.17g %.17g %d\n", p, pc.x1[k], pc.y1[k], pc.z1[k], pc.x2[k],
                    pc.y2[k], pc.z2[k], pc.portDirection[k]);
    }
    fclose(f);
    return 0;
}

int main(int argc, char **argv) {
    if (argc >= 5 && std::string(argv[1]) == "network") return network(argv[2], argv[3], argv[4]);
    if (argc >= 4 && std::string(argv[1]) == "simin") return simin(argv[2], argv[3]);
    fprintf(stderr, "usage: ref_network network <in> <out_dir> <design> | simin <file> <out>\n");
    return 1;
}
