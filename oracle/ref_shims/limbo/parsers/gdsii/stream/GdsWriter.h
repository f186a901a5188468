/* Project-written declaration stand-in for the GDSII writer that the
 * reference's limboint.hpp includes.  TEST INFRASTRUCTURE ONLY: the oracle
 * never writes GDSII; every member aborts if called. */
#pragma once
#include <cstdio>
#include <cstdlib>

namespace GdsParser {
class GdsWriter {
  public:
    explicit GdsWriter(const char *) {}
#define G2P_GDSW_STUB(name) \
    template <class... A> void name(A &&...) { std::fprintf(stderr, "GdsWriter::" #name " is not available\n"); std::abort(); }
    G2P_GDSW_STUB(create_lib) G2P_GDSW_STUB(gds_write_angle) G2P_GDSW_STUB(gds_write_aref) G2P_GDSW_STUB(gds_write_bgnstr)
    G2P_GDSW_STUB(gds_write_boundary) G2P_GDSW_STUB(gds_write_box) G2P_GDSW_STUB(gds_write_boxtype)
    G2P_GDSW_STUB(gds_write_colrow) G2P_GDSW_STUB(gds_write_datatype) G2P_GDSW_STUB(gds_write_endel)
    G2P_GDSW_STUB(gds_write_endlib) G2P_GDSW_STUB(gds_write_endstr) G2P_GDSW_STUB(gds_write_layer)
    G2P_GDSW_STUB(gds_write_mag) G2P_GDSW_STUB(gds_write_path) G2P_GDSW_STUB(gds_write_pathtype)
    G2P_GDSW_STUB(gds_write_presentation) G2P_GDSW_STUB(gds_write_sname) G2P_GDSW_STUB(gds_write_sref)
    G2P_GDSW_STUB(gds_write_strans) G2P_GDSW_STUB(gds_write_string) G2P_GDSW_STUB(gds_write_strname)
    G2P_GDSW_STUB(gds_write_text) G2P_GDSW_STUB(gds_write_texttype) G2P_GDSW_STUB(gds_write_width)
#undef G2P_GDSW_STUB
    // pointer form: callers pass variable-length arrays
    void gds_write_xy(const int *, const int *, size_t, bool = true) {
        std::fprintf(stderr, "GdsWriter::gds_write_xy is not available\n");
        std::abort();
    }
};
}  // namespace GdsParser
