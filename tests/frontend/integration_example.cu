// A reference-style program written against the front end: it must compile
// and link against the front-end headers and libmsl_gb300.so with the
// documented nvcc command line.
#include "muesli.h"
#include "dm.h"
using namespace msl;

MSL_USERFUNC float heat2D(const NPLMatrix<float> &m, int x, int y) {
    float v = 0;
    v += m(x - 1, y); v += m(x + 1, y); v += m(x, y - 1); v += m(x, y + 1);
    return v / 4;
}
int main(int argc, char **argv) {
    initSkeletons(argc, argv);
    DM<float> a(1024, 1024, 0, true), b(1024, 1024, 0, true);
    for (int i = 0; i < 100; i++) { a.mapStencil<heat2D>(b, 1, 0, false); b.mapStencil<heat2D>(a, 1, 0, false); }
    float *result = a.gather();
    terminateSkeletons();
}
