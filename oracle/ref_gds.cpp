/* Runs the reference's own GDSII database (AsciiDataBase) and saveToMesh
 * (limboint.hpp), compiled unmodified with the project's stream-reader
 * stand-in, on one GDSII file, and prints the conductor polygons that
 * saveToMesh leaves in fdtdMesh::conductorIn: one line per polygon,
 * "P layer nvert x0 y0 x1 y1 ..." (metres, %.17g); other lines are the
 * reference's own messages.  The top cell is the last
 * cell of the file, as the reference's command-line driver takes it.
 * TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.sh into oracle/_ref/.
 * usage: ref_gds <file.gds> [ignored GDSII layer ...] */
#include <cstdio>
#include <cstdlib>
#include "limboint.hpp"

int main(int argc, char **argv) {
    if (argc < 2) { fprintf(stderr, "usage: ref_gds <file.gds> [ignored layer ...]\n"); return 2; }
    AsciiDataBase adb;
    adb.setFileName(argv[1]);
    GdsParser::GdsReader rd(adb);
    if (!rd(argv[1])) { fprintf(stderr, "cannot read %s\n", argv[1]); return 3; }
    std::vector<int> ignore;
    for (int i = 2; i < argc; i++) ignore.push_back(atoi(argv[i]));
    fdtdMesh sys;
    const std::string top = adb.getCell(adb.getNumCell() - 1).getCellName();
    adb.saveToMesh(top, {0., 0.}, strans(), &sys, ignore);
    for (size_t i = 0; i < sys.conductorIn.size(); i++) {
        const fdtdOneCondct &c = sys.conductorIn[i];
        printf("P %d %d", (int)c.layer, (int)c.numVert);
        for (int v = 0; v < c.numVert; v++) printf(" %.17g %.17g", c.x[v], c.y[v]);
        printf("\n");
    }
    return 0;
}
