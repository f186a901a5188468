/* Project-written stand-in for the GDSII stream interface that the
 * reference's limboint.hpp includes (Limbo is not available here).  TEST
 * INFRASTRUCTURE ONLY: it lets the oracle compile the reference's own
 * AsciiDataBase and saveToMesh unmodified and drive them with records read
 * by a small reader of the GDSII stream format (record header: 2-byte length,
 * record type, data type; big-endian data).  The callbacks receive the
 * standard record names, signed 16/32-bit integers, decoded 8-byte reals
 * (excess-64, base 16) and strings cut at the first NUL, as the reference's
 * callbacks expect. */
#pragma once
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace GdsParser {

namespace GdsRecords {
enum EnumType {
    HEADER, BGNLIB, LIBNAME, UNITS, ENDLIB, BGNSTR, STRNAME, ENDSTR, BOUNDARY, PATH, SREF, AREF, TEXT, LAYER,
    DATATYPE, WIDTH, XY, ENDEL, SNAME, COLROW, TEXTNODE, NODE, TEXTTYPE, PRESENTATION, SPACING, STRING, STRANS,
    MAG, ANGLE, UINTEGER, USTRING, REFLIBS, FONTS, PATHTYPE, GENERATIONS, ATTRTABLE, STYPTABLE, STRTYPE, ELFLAGS,
    ELKEY, LINKTYPE, LINKKEYS, NODETYPE, PROPATTR, PROPVALUE, BOX, BOXTYPE, PLEX, BGNEXTN, ENDEXTN, TAPENUM,
    TAPECODE, STRCLASS, RESERVED, FORMAT, MASK, ENDMASKS, LIBDIRSIZE, SRFNAME, LIBSECUR, UNKNOWN
};
}
namespace GdsData {
enum EnumType { NO_DATA, BIT_ARRAY, INTEGER_2, INTEGER_4, REAL_4, REAL_8, STRING, UNKNOWN };
}

// String-keyed callbacks (what the reference's AsciiDataBase implements).
struct GdsDataBase {
    virtual ~GdsDataBase() {}
    virtual void bit_array_cbk(const char *, const char *, std::vector<int> const &) {}
    virtual void integer_2_cbk(const char *, const char *, std::vector<int> const &) {}
    virtual void integer_4_cbk(const char *, const char *, std::vector<int> const &) {}
    virtual void real_4_cbk(const char *, const char *, std::vector<double> const &) {}
    virtual void real_8_cbk(const char *, const char *, std::vector<double> const &) {}
    virtual void string_cbk(const char *, const char *, std::string const &) {}
    virtual void begin_end_cbk(const char *) {}
};

// Enum-keyed callbacks (declared for the reference's EnumDataBase; unused).
struct GdsDataBaseKernel {
    virtual ~GdsDataBaseKernel() {}
    virtual void bit_array_cbk(GdsRecords::EnumType, GdsData::EnumType, std::vector<int> const &) {}
    virtual void integer_2_cbk(GdsRecords::EnumType, GdsData::EnumType, std::vector<int> const &) {}
    virtual void integer_4_cbk(GdsRecords::EnumType, GdsData::EnumType, std::vector<int> const &) {}
    virtual void real_4_cbk(GdsRecords::EnumType, GdsData::EnumType, std::vector<double> const &) {}
    virtual void real_8_cbk(GdsRecords::EnumType, GdsData::EnumType, std::vector<double> const &) {}
    virtual void string_cbk(GdsRecords::EnumType, GdsData::EnumType, std::string const &) {}
    virtual void begin_end_cbk(GdsRecords::EnumType) {}
};

inline const char *gds_record_name(int t) {
    static const char *names[] = {
        "HEADER", "BGNLIB", "LIBNAME", "UNITS", "ENDLIB", "BGNSTR", "STRNAME", "ENDSTR", "BOUNDARY", "PATH", "SREF",
        "AREF", "TEXT", "LAYER", "DATATYPE", "WIDTH", "XY", "ENDEL", "SNAME", "COLROW", "TEXTNODE", "NODE",
        "TEXTTYPE", "PRESENTATION", "SPACING", "STRING", "STRANS", "MAG", "ANGLE", "UINTEGER", "USTRING",
        "REFLIBS", "FONTS", "PATHTYPE", "GENERATIONS", "ATTRTABLE", "STYPTABLE", "STRTYPE", "ELFLAGS", "ELKEY",
        "LINKTYPE", "LINKKEYS", "NODETYPE", "PROPATTR", "PROPVALUE", "BOX", "BOXTYPE", "PLEX", "BGNEXTN",
        "ENDEXTN", "TAPENUM", "TAPECODE", "STRCLASS", "RESERVED", "FORMAT", "MASK", "ENDMASKS", "LIBDIRSIZE",
        "SRFNAME", "LIBSECUR"};
    return t >= 0 && t < (int)(sizeof(names) / sizeof(names[0])) ? names[t] : "UNKNOWN";
}

// 8-byte GDSII real: sign, 7-bit excess-64 base-16 exponent, 56-bit fraction.
inline double gds_real8(const unsigned char *p) {
    uint64_t m = 0;
    for (int i = 1; i < 8; i++) m = (m << 8) | p[i];
    const int ex = (p[0] & 0x7f) - 64;
    const double v = std::ldexp((double)m, 4 * ex - 56);
    return (p[0] & 0x80) ? -v : v;
}

class GdsReader {
  public:
    explicit GdsReader(GdsDataBase &db) : db_(db) {}
    bool operator()(const char *filename) {
        FILE *f = std::fopen(filename, "rb");
        if (!f) return false;
        std::vector<unsigned char> b;
        unsigned char buf[65536];
        size_t n;
        while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) b.insert(b.end(), buf, buf + n);
        std::fclose(f);
        size_t o = 0;
        while (o + 4 <= b.size()) {
            const size_t len = ((size_t)b[o] << 8) | b[o + 1];
            if (len < 4 || o + len > b.size()) break;
            const int rt = b[o + 2], dt = b[o + 3];
            const unsigned char *d = &b[o + 4];
            const size_t nd = len - 4;
            const char *name = gds_record_name(rt);
            if (dt == 0) {
                db_.begin_end_cbk(name);
            } else if (dt == 1 || dt == 2) {
                std::vector<int> v;
                for (size_t i = 0; i + 1 < nd; i += 2) {
                    const int w = (d[i] << 8) | d[i + 1];
                    v.push_back(dt == 2 ? (int)(int16_t)w : w);
                }
                if (dt == 1) db_.bit_array_cbk(name, "BIT_ARRAY", v);
                else db_.integer_2_cbk(name, "INTEGER_2", v);
            } else if (dt == 3) {
                std::vector<int> v;
                for (size_t i = 0; i + 3 < nd; i += 4)
                    v.push_back((int)(int32_t)(((uint32_t)d[i] << 24) | ((uint32_t)d[i + 1] << 16) | ((uint32_t)d[i + 2] << 8) | d[i + 3]));
                db_.integer_4_cbk(name, "INTEGER_4", v);
            } else if (dt == 5) {
                std::vector<double> v;
                for (size_t i = 0; i + 7 < nd; i += 8) v.push_back(gds_real8(d + i));
                db_.real_8_cbk(name, "REAL_8", v);
            } else if (dt == 6) {
                std::string str;
                for (size_t i = 0; i < nd && d[i]; i++) str.push_back((char)d[i]);
                db_.string_cbk(name, "STRING", str);
            }
            o += len;
            if (rt == 4) break;   // ENDLIB
        }
        return true;
    }

  private:
    GdsDataBase &db_;
};

}  // namespace GdsParser
