// Test driver for include/gds2para_gb300_shim.hpp: the reference-signature
// generateStiff / paraGenerator / hypreSolve, instantiated with a mesh type
// that has the fdtdMesh members the shim reads and writes (src/fdtd.hpp:
// 182-356, with myint = long long as src/fdtd.hpp:30-36 defines it).
//
//   shim_driver extract <in_dir> <out_dir> <precision> <rtol>
//       reads the fdtdMesh fields written by tests/test_gpu_shim.py, calls
//       generateStiff then paraGenerator as TestMain.cpp:343,370 do, and
//       writes S_row/S_col/S_val, Z and whether the reference's frees
//       happened (freed.txt)
//   shim_driver hypre <in_dir> <out_dir>
//       reads A (row-sorted COO) and b, calls hypreSolve, writes x
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "gds2para_gb300_shim.hpp"

typedef long long myint;

struct ShimCdt {
    myint *node = nullptr;
    int markPort = 0;
};

struct ShimPort {
    int multiplicity = 0;
    std::vector<std::vector<myint>> portEdge;
    std::vector<double> portArea;
    std::vector<int> portDirection;
};

struct ShimMesh {
    double freqUnit = 1, freqStart = 0, freqEnd = 0;
    int nfreq = 1, freqScale = 1;
    double *xn = nullptr, *yn = nullptr, *zn = nullptr;
    myint N_cell_x = 0, N_cell_y = 0, N_cell_z = 0;
    std::vector<double> stackEpsn, stackSign;
    myint numCdt = 0;
    myint *markEdge = nullptr;
    ShimCdt *conductor = nullptr;
    myint *markNode = nullptr;
    myint *SRowId = nullptr, *SColId = nullptr;
    double *Sval = nullptr;
    myint leng_S = 0;
    std::vector<std::complex<double>> x;
    std::complex<double> *Y = nullptr;
    int numPorts = 0;
    std::vector<ShimPort> portCoor;
};

template <class T>
static std::vector<T> read_arr(const std::string &path) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) { std::fprintf(stderr, "cannot open %s\n", path.c_str()); std::exit(2); }
    const size_t bytes = (size_t)f.tellg();
    std::vector<T> v(bytes / sizeof(T));
    f.seekg(0);
    f.read(reinterpret_cast<char *>(v.data()), (std::streamsize)bytes);
    return v;
}

template <class T>
static T *malloc_copy(const std::vector<T> &v) {
    T *p = (T *)std::malloc(sizeof(T) * (v.size() ? v.size() : 1));
    for (size_t i = 0; i < v.size(); i++) p[i] = v[i];
    return p;
}

template <class T>
static void write_arr(const std::string &path, const T *p, size_t n) {
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char *>(p), (std::streamsize)(sizeof(T) * n));
}

static int extract(const std::string &in, const std::string &out, int precision, double rtol) {
    ShimMesh sys;
    {
        std::ifstream meta(in + "/meta.txt");
        myint nx, ny, nz;
        meta >> nx >> ny >> nz >> sys.numCdt >> sys.numPorts >> sys.nfreq >> sys.freqStart >> sys.freqEnd >>
            sys.freqUnit >> sys.freqScale;
        sys.N_cell_x = nx - 1; sys.N_cell_y = ny - 1; sys.N_cell_z = nz - 1;
    }
    sys.xn = malloc_copy(read_arr<double>(in + "/xn.f64"));
    sys.yn = malloc_copy(read_arr<double>(in + "/yn.f64"));
    sys.zn = malloc_copy(read_arr<double>(in + "/zn.f64"));
    sys.stackEpsn = read_arr<double>(in + "/stack_epsn.f64");
    sys.stackSign = read_arr<double>(in + "/stack_sign.f64");
    sys.markNode = malloc_copy(read_arr<myint>(in + "/mark_node.i64"));
    sys.markEdge = malloc_copy(read_arr<myint>(in + "/mark_edge.i64"));
    const std::vector<int32_t> mark_port = read_arr<int32_t>(in + "/mark_port.i32");
    sys.conductor = (ShimCdt *)std::calloc((size_t)(sys.numCdt ? sys.numCdt : 1), sizeof(ShimCdt));
    for (myint c = 0; c < sys.numCdt; c++) {
        sys.conductor[c].markPort = mark_port[c];
        sys.conductor[c].node = (myint *)std::malloc(sizeof(myint));   // freed by paraGenerator
    }
    const std::vector<int32_t> side_ptr = read_arr<int32_t>(in + "/port_side_ptr.i32");
    const std::vector<int64_t> edge_ptr = read_arr<int64_t>(in + "/side_edge_ptr.i64");
    const std::vector<int64_t> edges = read_arr<int64_t>(in + "/side_edges.i64");
    const std::vector<double> area = read_arr<double>(in + "/side_area.f64");
    const std::vector<int32_t> dir = read_arr<int32_t>(in + "/side_dir.i32");
    sys.portCoor.resize((size_t)sys.numPorts);
    for (int p = 0; p < sys.numPorts; p++) {
        ShimPort &pc = sys.portCoor[p];
        for (int s = side_ptr[p]; s < side_ptr[p + 1]; s++) {
            pc.multiplicity++;
            pc.portEdge.emplace_back(edges.begin() + edge_ptr[s], edges.begin() + edge_ptr[s + 1]);
            pc.portArea.push_back(area[s]);
            pc.portDirection.push_back(dir[s]);
        }
    }
    g2p_shim::settings().precision = precision;
    g2p_shim::settings().rtol = rtol;
    if (g2p_shim::generateStiff(&sys) != 0) return 3;
    write_arr(out + "/S_row.i64", sys.SRowId, (size_t)sys.leng_S);
    write_arr(out + "/S_col.i64", sys.SColId, (size_t)sys.leng_S);
    write_arr(out + "/S_val.f64", sys.Sval, (size_t)sys.leng_S);
    std::unordered_map<double, int> xi, yi, zi;
    if (g2p_shim::paraGenerator(&sys, xi, yi, zi) != 0) return 4;
    write_arr(out + "/Z.f64", reinterpret_cast<const double *>(sys.x.data()), 2 * sys.x.size());
    std::ofstream fr(out + "/freed.txt");
    fr << (sys.markNode == nullptr && sys.conductor == nullptr && sys.xn == nullptr && sys.yn == nullptr &&
           sys.zn == nullptr && sys.stackEpsn.empty() && sys.Y != nullptr)
       << "\n";
    std::free(sys.SRowId); std::free(sys.SColId); std::free(sys.Sval); std::free(sys.Y); std::free(sys.markEdge);
    return 0;
}

static int hypre(const std::string &in, const std::string &out) {
    std::vector<myint> r = read_arr<myint>(in + "/A_row.i64"), c = read_arr<myint>(in + "/A_col.i64");
    std::vector<double> v = read_arr<double>(in + "/A_val.f64"), b = read_arr<double>(in + "/b.f64");
    std::vector<double> x(b.size(), 0.0);
    ShimMesh *sys = nullptr;
    const int rc = g2p_shim::hypreSolve(sys, r.data(), c.data(), v.data(), (myint)v.size(), b.data(), (myint)b.size(),
                                        x.data());
    write_arr(out + "/x.f64", x.data(), x.size());
    return rc;
}

int main(int argc, char **argv) {
    if (argc >= 6 && std::string(argv[1]) == "extract") return extract(argv[2], argv[3], std::atoi(argv[4]), std::atof(argv[5]));
    if (argc >= 4 && std::string(argv[1]) == "hypre") return hypre(argv[2], argv[3]);
    std::fprintf(stderr, "usage: shim_driver extract <in> <out> <precision> <rtol> | hypre <in> <out>\n");
    return 1;
}
