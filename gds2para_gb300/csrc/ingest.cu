// Layout ingest, host code only:
//   * g2p_gdsii_read: reads a GDSII stream file and flattens its top cell
//     into the conductor polygons that the reference hands to its mesher
//     (fdtdMesh::conductorIn);
//   * g2p_mesh_grid: the mesher's grid lines from those polygons, the port
//     sides and the layer stack (below).
//
// The reference reads the stream with Limbo's parser into AsciiDataBase and
// flattens it with AsciiDataBase::saveToMesh (limboint.hpp:2823-3150, records
// at limboint.hpp:3413-3990, transforms at limboint.hpp:104-306, arrays at
// limboint.hpp:1535-1594).  This file restates that behaviour:
//   * coordinates, widths and begin extensions are scaled by the UNITS
//     record's metres per database unit;
//   * the end extension is never stored (the reference tests for a record
//     named ENDTEXTN, which does not exist), so it stays 0;
//   * boundaries and boxes are put in the reference's preferred order when
//     their element ends (see reorder), then keep every vertex but the
//     closing one; a box with a nonzero BOXTYPE is skipped; datatypes are
//     not checked;
//   * each path segment becomes a 4-vertex rectangle: a segment whose two x
//     coordinates are equal runs along y, every other one along x; the ends
//     of the first and last segment overshoot by half the width except for
//     PATHTYPE 0 (no overshoot) and 4 (2 * begin extension / width at the
//     start, the end extension 0 at the end); interior joints overshoot by
//     half the width; the corner order follows the segment's direction;
//   * STRANS resets magnification and angle, MAG and ANGLE (degrees) set
//     them; a point is mirrored in y, rotated, then magnified; nested
//     transforms compose by the reference's case table and wrap the angle to
//     [-pi, pi);
//   * an array reference places (cols - 1) x (rows - 1) instances at
//     p0 + i * colsep.x + j * rowsep.x in both coordinates;
//   * the top cell is the last cell of the file; references to unknown
//     cells are skipped.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

namespace {

struct Xform {
    bool mirror = false, abs_mag = false, abs_rot = false;
    double mag = 1.0, rot = 0.0;   // rot in radians

    // net transform of this one applied after `old` (the enclosing one)
    Xform after(const Xform &old) const {
        Xform t;
        t.mag = abs_mag ? mag : mag * old.mag;
        t.mirror = mirror != old.mirror;
        double r = rot;
        if (!abs_rot && old.rot != 0.) {
            if (!old.mirror && !mirror && rot == 0.) r = old.rot;
            else if (!old.mirror && !mirror) r += old.rot;
            else if (!old.mirror && mirror && rot == 0.) r = -1. * old.rot;
            else if (old.mirror && mirror && rot == 0.) r = -1. * old.rot;
            else if (old.mirror && !mirror && rot != 0.) r += old.rot;
            else if (mirror && rot != 0.) r -= old.rot;
        }
        t.rot = std::fmod(r + M_PI, 2. * M_PI) - M_PI;
        t.abs_mag = abs_mag;
        t.abs_rot = abs_rot;
        return t;
    }
    void apply(double x, double y, double &ox, double &oy) const {
        if (mirror) y = -y;
        if (rot != 0.) {
            const double wx = x, wy = y;
            x = +std::cos(rot) * wx + -std::sin(rot) * wy;
            y = +std::sin(rot) * wx + +std::cos(rot) * wy;
        }
        if (mag != 1.) { x *= mag; y *= mag; }
        ox = x;
        oy = y;
    }
};

struct Shape {              // boundary, box or path
    int layer = 0, type = 0;
    double width = 0., bext = 0.;
    std::vector<double> xy;
};
struct Ref {
    std::string name;
    Xform t;
    int cols = 0, rows = 0;
    std::vector<double> xy;
};
struct Cell {
    std::string name;
    std::vector<Shape> bounds, paths, boxes;
    std::vector<Ref> srefs, arefs;
};

// The order boundaries and boxes are stored in once their element ends
// (limboint.hpp:453-496, 1031-1075): a closing point equal to the first is
// dropped, the list is rotated to start at the lower-right point found by
// the reference's scan (x >= and y <= the current pick), reversed after its
// first point when that first step goes left and not up, then closed again.
void reorder(std::vector<double> &v) {
    size_t n = v.size() / 2;
    if (n < 2) return;
    if (v[0] == v[2 * (n - 1)] && v[1] == v[2 * (n - 1) + 1]) {
        v.pop_back();
        v.pop_back();
        n--;
    }
    if (n < 2) return;
    size_t lr = 0;
    for (size_t i = 1; i < n; i++)
        if (v[2 * i] >= v[2 * lr] && v[2 * i + 1] <= v[2 * lr + 1]) lr = i;
    std::rotate(v.begin(), v.begin() + 2 * lr, v.end());
    if (v[0] > v[2] && v[1] >= v[3]) {
        std::vector<double> r = {v[0], v[1]};
        for (size_t i = n - 1; i > 0; i--) { r.push_back(v[2 * i]); r.push_back(v[2 * i + 1]); }
        v = r;
    }
    v.push_back(v[0]);
    v.push_back(v[1]);
}

double real8(const unsigned char *p) {
    uint64_t m = 0;
    for (int i = 1; i < 8; i++) m = (m << 8) | p[i];
    const double v = std::ldexp((double)m, 4 * ((p[0] & 0x7f) - 64) - 56);
    return (p[0] & 0x80) ? -v : v;
}

bool parse(const std::vector<unsigned char> &b, std::vector<Cell> &cells) {
    enum { NONE, BOUND, PATH, BOX, SREF, AREF, OTHER } el = NONE;
    double unit = 0.0;   // metres per database unit
    size_t o = 0;
    while (o + 4 <= b.size()) {
        const size_t len = ((size_t)b[o] << 8) | b[o + 1];
        if (len < 4 || o + len > b.size()) return false;
        const int rt = b[o + 2], dt = b[o + 3];
        const unsigned char *d = &b[o + 4];
        const size_t nd = len - 4;
        std::vector<int> iv;
        if (dt == 1 || dt == 2)
            for (size_t i = 0; i + 1 < nd; i += 2) {
                const int w = (d[i] << 8) | d[i + 1];
                iv.push_back(dt == 2 ? (int)(int16_t)w : w);
            }
        else if (dt == 3)
            for (size_t i = 0; i + 3 < nd; i += 4)
                iv.push_back((int)(int32_t)(((uint32_t)d[i] << 24) | ((uint32_t)d[i + 1] << 16) | ((uint32_t)d[i + 2] << 8) | d[i + 3]));
        std::vector<double> rv;
        if (dt == 5)
            for (size_t i = 0; i + 7 < nd; i += 8) rv.push_back(real8(d + i));
        std::string str;
        if (dt == 6)
            for (size_t i = 0; i < nd && d[i]; i++) str.push_back((char)d[i]);
        Cell *c = cells.empty() ? nullptr : &cells.back();
        Shape *sh = !c ? nullptr : el == BOUND ? (c->bounds.empty() ? nullptr : &c->bounds.back())
                               : el == PATH  ? (c->paths.empty() ? nullptr : &c->paths.back())
                               : el == BOX   ? (c->boxes.empty() ? nullptr : &c->boxes.back()) : nullptr;
        Ref *rf = !c ? nullptr : el == SREF ? (c->srefs.empty() ? nullptr : &c->srefs.back())
                             : el == AREF ? (c->arefs.empty() ? nullptr : &c->arefs.back()) : nullptr;
        switch (rt) {
        case 0x03: if (rv.size() >= 2) unit = rv[1]; break;                            // UNITS
        case 0x05: cells.emplace_back(); el = NONE; break;                              // BGNSTR
        case 0x06: if (c) c->name = str; break;                                         // STRNAME
        case 0x08: if (c) { c->bounds.emplace_back(); el = BOUND; } break;              // BOUNDARY
        case 0x09: if (c) { c->paths.emplace_back(); c->paths.back().type = 2; el = PATH; } break;   // PATH
        case 0x2D: if (c) { c->boxes.emplace_back(); el = BOX; } break;                 // BOX
        case 0x0A: if (c) { c->srefs.emplace_back(); el = SREF; } break;                // SREF
        case 0x0B: if (c) { c->arefs.emplace_back(); el = AREF; } break;                // AREF
        case 0x0C: case 0x15: el = OTHER; break;                                        // TEXT, NODE
        case 0x0D: if (sh && !iv.empty()) sh->layer = iv[0]; break;                     // LAYER
        case 0x21: if (el == PATH && sh && !iv.empty()) sh->type = iv[0]; break;        // PATHTYPE
        case 0x2E: if (el == BOX && sh && !iv.empty()) sh->type = iv[0]; break;         // BOXTYPE
        case 0x0F: if (el == PATH && sh && !iv.empty()) sh->width = unit * iv[0]; break;    // WIDTH
        case 0x30: if (el == PATH && sh && !iv.empty()) sh->bext = unit * iv[0]; break;     // BGNEXTN
        case 0x10:                                                                      // XY
            if (sh || rf) {
                std::vector<double> &xy = sh ? sh->xy : rf->xy;
                xy.clear();
                for (int v : iv) xy.push_back(unit * v);
            }
            break;
        case 0x12: if (rf) rf->name = str; break;                                       // SNAME
        case 0x13: if (el == AREF && rf && iv.size() >= 2) { rf->cols = iv[0]; rf->rows = iv[1]; } break;   // COLROW
        case 0x1A:                                                                      // STRANS
            if (rf && !iv.empty()) {
                rf->t = Xform();
                rf->t.mirror = (iv[0] & 0x8000) != 0;
                rf->t.abs_mag = (iv[0] & 0x4) != 0;
                rf->t.abs_rot = (iv[0] & 0x2) != 0;
            }
            break;
        case 0x1B: if (rf && !rv.empty()) rf->t.mag = rv[0]; break;                     // MAG
        case 0x1C: if (rf && !rv.empty()) rf->t.rot = M_PI / 180. * rv[0]; break;       // ANGLE
        case 0x11:                                                                      // ENDEL
            if ((el == BOUND || el == BOX) && sh) reorder(sh->xy);
            el = NONE;
            break;
        default: break;
        }
        o += len;
        if (rt == 0x04) break;   // ENDLIB
    }
    return true;
}

struct Flat {
    std::vector<int32_t> layer;
    std::vector<int64_t> vptr{0};
    std::vector<double> x, y;
};

bool ignored(int layer, const std::vector<int> &ign) {
    for (int l : ign) if (l == layer) return true;
    return false;
}

void flatten(const std::vector<Cell> &cells, const std::string &name, double xo, double yo, const Xform &t,
             const std::vector<int> &ign, Flat &out, int depth) {
    size_t ci = 0;
    while (ci < cells.size() && cells[ci].name != name) ci++;
    if (ci == cells.size() || depth > 64) return;
    const Cell &c = cells[ci];
    auto put = [&](double px, double py) {
        double ox, oy;
        t.apply(px, py, ox, oy);
        out.x.push_back(ox + xo);
        out.y.push_back(oy + yo);
    };
    auto close = [&](int layer) {
        out.layer.push_back(layer);
        out.vptr.push_back((int64_t)out.x.size());
    };
    for (const Shape &s : c.bounds) {
        if (ignored(s.layer, ign) || s.xy.size() < 4) continue;
        for (size_t j = 0; j + 2 < s.xy.size(); j += 2) put(s.xy[j], s.xy[j + 1]);
        close(s.layer);
    }
    for (const Shape &s : c.paths) {
        if (ignored(s.layer, ign) || s.xy.size() < 4) continue;
        const double w = s.width, h = w / 2.;
        const std::vector<double> &p = s.xy;
        for (size_t j = 0; j + 2 < p.size(); j += 2) {
            double o1 = 1.0, o2 = 1.0;
            if (j == 0) { if (s.type == 0) o1 = 0.0; else if (s.type == 4) o1 = 2. / w * s.bext; }
            if (j == p.size() - 4) { if (s.type == 0) o2 = 0.0; else if (s.type == 4) o2 = 2. / w * 0.0; }
            const double x1 = p[j], y1 = p[j + 1], x2 = p[j + 2], y2 = p[j + 3];
            if (x1 == x2) {            // along y
                if (y1 > y2) {
                    put(x1 - h, y1 + o1 * h); put(x1 + h, y1 + o1 * h); put(x2 + h, y2 - o2 * h); put(x2 - h, y2 - o2 * h);
                } else {
                    put(x1 - h, y1 - o1 * h); put(x1 + h, y1 - o1 * h); put(x2 + h, y2 + o2 * h); put(x2 - h, y2 + o2 * h);
                }
            } else {                   // along x
                if (x1 > x2) {
                    put(x1 + o1 * h, y1 + h); put(x1 + o1 * h, y1 - h); put(x2 - o2 * h, y2 - h); put(x2 - o2 * h, y2 + h);
                } else {
                    put(x1 - o1 * h, y1 + h); put(x1 - o1 * h, y1 - h); put(x2 + o2 * h, y2 - h); put(x2 + o2 * h, y2 + h);
                }
            }
            close(s.layer);
        }
    }
    for (const Shape &s : c.boxes) {
        if (s.type != 0 || ignored(s.layer, ign) || s.xy.size() < 4) continue;
        for (size_t j = 0; j + 2 < s.xy.size(); j += 2) put(s.xy[j], s.xy[j + 1]);
        close(s.layer);
    }
    for (const Ref &r : c.srefs) {
        if (r.xy.size() != 2) continue;
        double px, py;
        t.apply(r.xy[0], r.xy[1], px, py);
        flatten(cells, r.name, px + xo, py + yo, r.t.after(t), ign, out, depth + 1);
    }
    for (const Ref &r : c.arefs) {
        if (r.xy.size() < 6) continue;
        const double cx = r.cols >= 2 ? (r.xy[2] - r.xy[0]) / (r.cols - 1.) : 0.;
        const double rx = r.rows >= 2 ? (r.xy[4] - r.xy[0]) / (r.rows - 1.) : 0.;
        for (int i = 0; i < r.cols - 1; i++)
            for (int j = 0; j < r.rows - 1; j++) {
                const double ix = r.xy[0] + i * cx + j * rx + 0., iy = r.xy[1] + i * cx + j * rx + 0.;
                double px, py;
                t.apply(ix, iy, px, py);
                flatten(cells, r.name, px + xo, py + yo, r.t.after(t), ign, out, depth + 1);
            }
    }
}

}  // namespace

struct g2p_polygons {
    Flat f;
};

extern "C" g2p_status g2p_gdsii_read(const char *path, const int32_t *ignore_layers, int32_t n_ignore,
                                     g2p_polygons **out) {
    if (!path || !out || n_ignore < 0 || (n_ignore > 0 && !ignore_layers)) {
        g2p::set_last_message("bad arguments");
        return G2P_ERR_INVALID;
    }
    *out = nullptr;
    FILE *fp = std::fopen(path, "rb");
    if (!fp) { g2p::set_last_message("cannot open %s", path); return G2P_ERR_INVALID; }
    std::vector<unsigned char> b;
    unsigned char buf[65536];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, fp)) > 0) b.insert(b.end(), buf, buf + n);
    std::fclose(fp);
    try {
        std::vector<Cell> cells;
        if (!parse(b, cells) || cells.empty()) {
            g2p::set_last_message("%s: not a GDSII stream with a cell", path);
            return G2P_ERR_INVALID;
        }
        std::vector<int> ign(ignore_layers, ignore_layers + n_ignore);
        auto *p = new g2p_polygons();
        flatten(cells, cells.back().name, 0., 0., Xform(), ign, p->f, 0);
        *out = p;
    } catch (const std::exception &e) {
        g2p::set_last_message("GDSII read: %s", e.what());
        return G2P_ERR_INVALID;
    }
    return G2P_OK;
}

extern "C" g2p_status g2p_polygons_size(const g2p_polygons *p, int64_t *npoly, int64_t *nvert) {
    if (!p || !npoly || !nvert) { g2p::set_last_message("bad arguments"); return G2P_ERR_INVALID; }
    *npoly = (int64_t)p->f.layer.size();
    *nvert = (int64_t)p->f.x.size();
    return G2P_OK;
}

extern "C" g2p_status g2p_polygons_get(const g2p_polygons *p, int32_t *layer, int64_t *vert_ptr, double *x, double *y) {
    if (!p || !layer || !vert_ptr || !x || !y) { g2p::set_last_message("bad arguments"); return G2P_ERR_INVALID; }
    std::memcpy(layer, p->f.layer.data(), sizeof(int32_t) * p->f.layer.size());
    std::memcpy(vert_ptr, p->f.vptr.data(), sizeof(int64_t) * p->f.vptr.size());
    std::memcpy(x, p->f.x.data(), sizeof(double) * p->f.x.size());
    std::memcpy(y, p->f.y.data(), sizeof(double) * p->f.y.size());
    return G2P_OK;
}

extern "C" void g2p_polygons_free(g2p_polygons *p) { delete p; }

// ------------------------------------------------------------ grid lines
// The grid of the reference's meshAndMark (mesh.cpp:5-330), restated:
//   * x (and y) candidates are every polygon vertex and both ends of every
//     port side, sorted.  Walking them with `last` the last coordinate
//     accepted: a candidate more than disMin but at most disMax from `last`
//     is kept and becomes `last`; one more than disMax away first gets lines
//     every disMax from the previous line until within disMax, becomes
//     `last` only if still more than disMin away, and is kept; any other is
//     kept without moving `last`.  The kept lines are sorted again and every
//     line within disMin of the last one kept is merged away.
//     disMin = 1e-3 * min(x extent, y extent), disMax = 0.005 * extent.
//   * z candidates are both ends of every stack layer and of every port
//     side; a sorted candidate within 0.05 * (thinnest layer, or the z
//     extent) of the previous candidate is merged away.
//   * each cell layer takes eps and sigma of the stack layer that contains
//     its midpoint, scanning layers upward from the first when the first
//     layer starts at the lowest line and downward from the last otherwise;
//     one more entry repeats the last layer found (the top surface).
namespace {
constexpr double kMaxGridLines = 67108864.0;   // 2^26 lines per axis

// The fill loop gives up once more than `cap` lines have been placed and sets
// *over (a guard: the caller sizes `cap` from the vertex span, which bounds
// the fill).
std::vector<double> axis_lines(std::vector<double> o, double dmin, double dmax, int64_t cap, bool *over) {
    std::sort(o.begin(), o.end());
    std::vector<double> v{o[0]};
    double last = o[0];
    for (size_t i = 1; i < o.size(); i++) {
        const double d = std::fabs(o[i] - last);
        if (d > dmin && d <= dmax) {
            v.push_back(o[i]);
            last = o[i];
        } else if (d > dmin) {
            while (std::fabs(o[i] - last) > dmax) {
                if ((int64_t)v.size() > cap) { *over = true; return v; }
                v.push_back(v.back() + dmax);
                last = v.back();
            }
            if (std::fabs(o[i] - last) > dmin) last = o[i];
            v.push_back(o[i]);
        } else {
            v.push_back(o[i]);
        }
    }
    std::sort(v.begin(), v.end());
    std::vector<double> out{v[0]};
    last = v[0];
    for (size_t i = 1; i < v.size(); i++)
        if (std::fabs(v[i] - last) > dmin) { out.push_back(v[i]); last = v[i]; }
    return out;
}
}  // namespace

extern "C" g2p_status g2p_mesh_grid(const double *lim, int64_t npoly, const int64_t *vert_ptr, const double *vx,
                                    const double *vy, int32_t nside, const double *sides, int32_t nstack,
                                    const double *stack, int64_t cap_xy, int64_t cap_z, double *xn, double *yn,
                                    double *zn, double *stack_epsn, double *stack_sign, int64_t *counts) {
    if (!lim || npoly < 0 || nside < 0 || nstack < 1 || !stack || !counts || (npoly > 0 && (!vert_ptr || !vx || !vy)) ||
        (nside > 0 && !sides)) {
        g2p::set_last_message("bad arguments");
        return G2P_ERR_INVALID;
    }
    try {
        std::vector<double> ox, oy, oz;
        const int64_t nv = npoly > 0 ? vert_ptr[npoly] : 0;
        for (int64_t i = 0; i < nv; i++) { ox.push_back(vx[i]); oy.push_back(vy[i]); }
        for (int32_t k = 0; k < nside; k++) {
            const double *c = sides + 6 * (int64_t)k;
            ox.push_back(c[0]); oy.push_back(c[1]);
            ox.push_back(c[3]); oy.push_back(c[4]);
        }
        if (ox.empty()) { g2p::set_last_message("no polygon vertices or port sides"); return G2P_ERR_INVALID; }
        for (int k = 0; k < 6; k++)
            if (!std::isfinite(lim[k])) { g2p::set_last_message("layout limits must be finite"); return G2P_ERR_INVALID; }
        if (!(lim[1] > lim[0]) || !(lim[3] > lim[2])) {
            g2p::set_last_message("layout limits need xlim2 > xlim1 and ylim2 > ylim1 (got %g..%g, %g..%g)", lim[0],
                                  lim[1], lim[2], lim[3]);
            return G2P_ERR_INVALID;
        }
        double minlayer = lim[5] - lim[4];
        for (int32_t k = 0; k < nstack; k++) {
            const double b = stack[4 * k], e = stack[4 * k + 1];
            oz.push_back(b);
            oz.push_back(e);
            if (e - b > 0) minlayer = std::fmin(minlayer, e - b);
        }
        for (int32_t k = 0; k < nside; k++) { oz.push_back(sides[6 * k + 2]); oz.push_back(sides[6 * k + 5]); }
        const double dmin = 1e-3 * std::fmin(lim[3] - lim[2], lim[1] - lim[0]);
        // Each axis gets at most (vertex span / disMax) fill lines besides its
        // candidates; a span that would need more than 2^26 lines is refused
        // before any is placed.
        auto fill_bound = [](const std::vector<double> &o, double dmax) {
            const auto mm = std::minmax_element(o.begin(), o.end());
            return (*mm.second - *mm.first) / dmax + (double)o.size() + 1;
        };
        const double dmax_x = 0.005 * (lim[1] - lim[0]), dmax_y = 0.005 * (lim[3] - lim[2]);
        const double bx = fill_bound(ox, dmax_x), by = fill_bound(oy, dmax_y);
        if (!(bx < kMaxGridLines) || !(by < kMaxGridLines)) {
            g2p::set_last_message("grid would need more than %lld lines along %s: the vertices span far more than "
                                  "the layout limits", (long long)kMaxGridLines, bx < kMaxGridLines ? "y" : "x");
            return G2P_ERR_INVALID;
        }
        bool over_x = false, over_y = false;
        const std::vector<double> gx = axis_lines(ox, dmin, dmax_x, (int64_t)bx, &over_x);
        const std::vector<double> gy = axis_lines(oy, dmin, dmax_y, (int64_t)by, &over_y);
        if (over_x || over_y) {
            g2p::set_last_message("grid fill along %s exceeded its bound", over_x ? "x" : "y");
            return G2P_ERR_INVALID;
        }
        std::sort(oz.begin(), oz.end());
        const double dminz = minlayer * 0.05;
        std::vector<double> gz{oz[0]};
        for (size_t i = 1; i < oz.size(); i++)
            if (std::fabs(oz[i] - oz[i - 1]) > dminz) gz.push_back(oz[i]);
        const int64_t nz = (int64_t)gz.size();
        std::vector<double> eps, sig;
        const bool up = stack[0] == gz[0];
        int32_t j = up ? 0 : nstack - 1;
        for (int64_t i = 0; i < nz - 1;) {
            if (j < 0 || j >= nstack) { g2p::set_last_message("grid layer %lld lies in no stack layer", (long long)i); return G2P_ERR_INVALID; }
            const double mid = (gz[i] + gz[i + 1]) / 2;
            if (mid >= stack[4 * j] && mid <= stack[4 * j + 1]) {
                eps.push_back(stack[4 * j + 2]);
                sig.push_back(stack[4 * j + 3]);
                i++;
            } else {
                j += up ? 1 : -1;
            }
        }
        if (j < 0 || j >= nstack) { g2p::set_last_message("top surface lies in no stack layer"); return G2P_ERR_INVALID; }
        eps.push_back(stack[4 * j + 2]);
        sig.push_back(stack[4 * j + 3]);
        counts[0] = (int64_t)gx.size();
        counts[1] = (int64_t)gy.size();
        counts[2] = nz;
        if (counts[0] > cap_xy || counts[1] > cap_xy || nz > cap_z || !xn || !yn || !zn || !stack_epsn || !stack_sign) {
            g2p::set_last_message("grid needs %lld x %lld x %lld lines", (long long)counts[0], (long long)counts[1],
                                  (long long)nz);
            return G2P_ERR_INVALID;
        }
        std::copy(gx.begin(), gx.end(), xn);
        std::copy(gy.begin(), gy.end(), yn);
        std::copy(gz.begin(), gz.end(), zn);
        std::copy(eps.begin(), eps.end(), stack_epsn);
        std::copy(sig.begin(), sig.end(), stack_sign);
    } catch (const std::exception &e) {
        g2p::set_last_message("grid: %s", e.what());
        return G2P_ERR_INVALID;
    }
    return G2P_OK;
}

// ---------------------------------------------------------------------------
// .sim_input reader: the reference's SolverDataBase::readSimInput
// (src/solnoutclass.hpp:5412-5886) followed by what convertToFDTDMesh takes
// from it (src/solnoutclass.hpp:5894-5984): the limits and length unit, the
// frequency sweep, the physically valid stack layers (height > 0, eps_r >= 1,
// sigma >= 0) with their GDSII numbers, and the ports with their sides and
// each side's current direction (Port::positiveCoordFlow: +1 when a supply
// coordinate exceeds the return's).
//
// The text rules are the reference's: a section starts at a line beginning
// "TOTAL SIZE", "FREQUENCY", "DIELECTRIC STACK" or "PORT"; lines starting
// with '#' are skipped inside a section; values follow "key = "; a port line
// is told apart by its count of spaces before " #" (4: x y x y GDSII-layer,
// the z range that layer's; 6: six coordinates and the direction; more: a
// name first), sides with the same name make one port, and unnamed lines are
// all named "port1" (the reference never advances that counter); a stack
// layer's GDSII number is its name, or the digits after an 'M' in it; a
// missing "z = " continues from the layer below.  Like the reference, the
// line loop stops at the end of the file, so a last line without a newline
// is not read.
namespace {

struct SimLayer {
    std::string name;
    int gdsii;
    double z, h, eps, sigma;
    bool valid() const { return h > 0.0 && eps >= 1.0 && sigma >= 0.0; }
};

struct SimPort {
    std::string name;
    std::vector<double> coord;   // 6 per side
};

// stod of the text after position `at`, as the reference's
// stod(line.substr(at, ...)) reads it; false when no number is there
bool num_at(const std::string &line, size_t at, double *v) {
    if (at == std::string::npos || at > line.size()) return false;
    const char *b = line.c_str() + at;
    char *e = nullptr;
    *v = strtod(b, &e);
    return e != b;
}

}  // namespace

struct g2p_sim_input {
    double lim[6] = {0, 0, 0, 0, 0, 0};
    double length_unit = 1, freq_unit = 1, freq_start = 0, freq_end = 0;
    int32_t nfreq = 1, freq_scale = 1;
    std::vector<SimLayer> layers;
    std::vector<SimPort> ports;
};

extern "C" g2p_status g2p_sim_input_read(const char *path, g2p_sim_input **out) {
    if (!path || !out) { g2p::set_last_message("g2p_sim_input_read: null argument"); return G2P_ERR_INVALID; }
    FILE *f = fopen(path, "rb");
    if (!f) { g2p::set_last_message("g2p_sim_input_read: cannot open %s", path); return G2P_ERR_INVALID; }
    std::string text;
    char buf[65536];
    for (size_t n; (n = fread(buf, 1, sizeof buf, f)) > 0;) text.append(buf, n);
    fclose(f);
    // std::getline over the text: each call returns the next line and
    // reports the end of the file when it ran into it
    size_t pos = 0;
    bool eof = false;
    auto getline = [&](std::string &line) {
        line.clear();
        if (pos >= text.size()) { eof = true; return; }
        const size_t nl = text.find('\n', pos);
        if (nl == std::string::npos) { line = text.substr(pos); pos = text.size(); eof = true; return; }
        line = text.substr(pos, nl - pos);
        pos = nl + 1;
    };
    auto skip_comments = [&](std::string &line) {
        while (line.compare(0, 1, "#") == 0 && !eof) getline(line);
    };
    auto value_after = [](const std::string &line, const char *key, double *v) {
        const size_t at = line.find(key);
        return at != std::string::npos && num_at(line, at + strlen(key), v);
    };
    auto bad = [&](const char *what) {
        g2p::set_last_message("g2p_sim_input_read: %s: %s", path, what);
        return G2P_ERR_INVALID;
    };
    g2p_sim_input r;
    std::string line;
    getline(line);
    while (!eof) {
        if (line.compare(0, 10, "TOTAL SIZE") == 0) {
            getline(line);
            skip_comments(line);
            const std::string nc = line.substr(0, line.find(" #"));
            if (std::count(nc.begin(), nc.end(), ' ') < 5) {
                g2p::set_last_message("g2p_sim_input_read: %s: a board outline file in place of the x/y limits is not "
                                 "supported", path);
                return G2P_ERR_UNSUPPORTED;
            }
            double v[6];
            size_t at = 0;
            for (int k = 0; k < 6; k++) {
                if (!num_at(line, at, &v[k])) return bad("TOTAL SIZE limits");
                at = line.find(' ', at);
                if (k < 5 && at == std::string::npos) return bad("TOTAL SIZE limits");
                at += 1;
            }
            getline(line);
            skip_comments(line);
            if (!value_after(line, "lengthUnit = ", &r.length_unit)) return bad("lengthUnit");
            for (int k = 0; k < 6; k++) r.lim[k] = v[k] * r.length_unit;
        } else if (line.compare(0, 9, "FREQUENCY") == 0) {
            double nf = 0, fs = 0;
            const char *keys[5] = {"freqUnit = ", "freqStart = ", "freqEnd = ", "nfreq = ", "freqScale = "};
            double *dst[5] = {&r.freq_unit, &r.freq_start, &r.freq_end, &nf, &fs};
            for (int k = 0; k < 5; k++) {
                getline(line);
                skip_comments(line);
                if (!value_after(line, keys[k], dst[k])) return bad(keys[k]);
            }
            r.nfreq = (int32_t)nf;
            r.freq_scale = (int32_t)fs;
            if (r.nfreq < 1) return bad("nfreq");
            // convertToFDTDMesh takes the first and last of the frequency
            // list, which holds freqStart alone for one point
            if (r.nfreq == 1) r.freq_end = r.freq_start;
        } else if (line.compare(0, 16, "DIELECTRIC STACK") == 0) {
            getline(line);
            skip_comments(line);
            double ns = 0;
            if (!value_after(line, "numStack = ", &ns) && !value_after(line, "numLayer = ", &ns)) ns = 0;
            getline(line);
            skip_comments(line);
            for (int64_t k = 0; k < (int64_t)ns; k++) {
                SimLayer L;
                L.name = line.substr(0, line.find(' '));
                L.gdsii = -1;
                const size_t m = L.name.find('M');
                const std::string digits = m != std::string::npos ? L.name.substr(m + 1) : L.name;
                if (!digits.empty() && std::all_of(digits.begin(), digits.end(), [](char c) { return c >= '0' && c <= '9'; }))
                    L.gdsii = atoi(digits.c_str());
                if (line.find("z = ") != std::string::npos) {
                    if (!value_after(line, "z = ", &L.z)) return bad("stack layer z");
                    L.z *= r.length_unit;
                } else {
                    L.z = r.layers.empty() ? 0.0 : r.layers.back().z + r.layers.back().h;
                }
                if (!value_after(line, "h = ", &L.h) || !value_after(line, "e = ", &L.eps)) return bad("stack layer h or e");
                L.h *= r.length_unit;
                L.sigma = 0.;
                if (line.find("sigma = ") != std::string::npos && !value_after(line, "sigma = ", &L.sigma))
                    return bad("stack layer sigma");
                r.layers.push_back(L);
                getline(line);
                skip_comments(line);
            }
        } else if (line.compare(0, 4, "PORT") == 0 && r.ports.empty()) {
            getline(line);
            skip_comments(line);
            getline(line);
            skip_comments(line);
            while (line.size() >= 3 && !eof) {
                const std::string nc = line.substr(0, line.find(" #"));
                const size_t nsp = (size_t)std::count(nc.begin(), nc.end(), ' ');
                std::string name;
                double c[6];
                std::vector<double> vals;
                size_t at = 0;
                auto next_num = [&](double *v) {
                    if (!num_at(line, at, v)) return false;
                    at = line.find(' ', at);
                    at = at == std::string::npos ? line.size() : at + 1;
                    return true;
                };
                if (nsp == 4) {
                    double xs, ys, xr, yr, lay;
                    if (!next_num(&xs) || !next_num(&ys) || !next_num(&xr) || !next_num(&yr) || !next_num(&lay))
                        return bad("port line");
                    const SimLayer *L = nullptr;
                    for (const auto &l : r.layers)
                        if (l.gdsii == (int)lay) { L = &l; break; }
                    if (!L) return bad("port layer not in the stack");
                    name = "port1";
                    const double u = r.length_unit;
                    const double cc[6] = {xs * u, ys * u, L->z, xr * u, yr * u, L->z + L->h};
                    std::copy(cc, cc + 6, c);
                } else if (nsp >= 6) {
                    if (nsp > 6) {
                        const size_t sp = line.find(' ');
                        name = line.substr(0, sp);
                        at = sp + 1;
                    } else {
                        name = "port1";
                    }
                    for (int k = 0; k < 6; k++) {
                        if (!next_num(&c[k])) return bad("port line");
                        c[k] *= r.length_unit;
                    }
                    double dir;
                    if (!next_num(&dir)) return bad("port line direction");
                } else {
                    return bad("port line");
                }
                SimPort *P = nullptr;
                for (auto &p : r.ports)
                    if (p.name == name) { P = &p; break; }
                if (!P) { r.ports.push_back(SimPort{name, {}}); P = &r.ports.back(); }
                P->coord.insert(P->coord.end(), c, c + 6);
                getline(line);
                while (line.compare(0, 1, "#") == 0 && !eof) getline(line);
            }
        }
        getline(line);
    }
    *out = new g2p_sim_input(r);
    return G2P_OK;
}

extern "C" g2p_status g2p_sim_input_sizes(const g2p_sim_input *s, int32_t *nlayer, int32_t *nport, int32_t *nside) {
    if (!s || !nlayer || !nport || !nside) return G2P_ERR_INVALID;
    int32_t nl = 0, ns = 0;
    for (const auto &l : s->layers) nl += l.valid() ? 1 : 0;
    for (const auto &p : s->ports) ns += (int32_t)(p.coord.size() / 6);
    *nlayer = nl;
    *nport = (int32_t)s->ports.size();
    *nside = ns;
    return G2P_OK;
}

extern "C" g2p_status g2p_sim_input_get(const g2p_sim_input *s, double *lim, double *units, int32_t *freq_counts,
                                        double *layers, int32_t *layer_gdsii, int32_t *port_side_ptr,
                                        double *side_coords, int32_t *side_dir) {
    if (!s) return G2P_ERR_INVALID;
    if (lim) std::copy(s->lim, s->lim + 6, lim);
    if (units) {
        units[0] = s->length_unit;
        units[1] = s->freq_unit;
        units[2] = s->freq_start;
        units[3] = s->freq_end;
    }
    if (freq_counts) { freq_counts[0] = s->nfreq; freq_counts[1] = s->freq_scale; }
    int64_t k = 0;
    for (const auto &l : s->layers) {
        if (!l.valid()) continue;
        if (layers) {
            layers[4 * k] = l.z;
            layers[4 * k + 1] = l.z + l.h;
            layers[4 * k + 2] = l.eps;
            layers[4 * k + 3] = l.sigma;
        }
        if (layer_gdsii) layer_gdsii[k] = l.gdsii;
        k++;
    }
    int32_t side = 0;
    if (port_side_ptr) port_side_ptr[0] = 0;
    for (size_t p = 0; p < s->ports.size(); p++) {
        const auto &c = s->ports[p].coord;
        for (size_t q = 0; q + 6 <= c.size(); q += 6, side++) {
            if (side_coords) std::copy(c.begin() + q, c.begin() + q + 6, side_coords + 6 * (int64_t)side);
            if (side_dir) side_dir[side] = (c[q] > c[q + 3] || c[q + 1] > c[q + 4] || c[q + 2] > c[q + 5]) ? 1 : -1;
        }
        if (port_side_ptr) port_side_ptr[p + 1] = side;
    }
    return G2P_OK;
}

extern "C" void g2p_sim_input_free(g2p_sim_input *s) { delete s; }
