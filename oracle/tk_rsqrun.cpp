// tk_rsqrun.cpp -- runs the reference's own rsq reader (FBPG/rsq_load.cpp,
// class rsq) through its public interface: LoadImages(first, last), then
// ProccessAndCopy, which applies FlatFieldCorrection (rsq_load.cpp:299-325)
// and, per the settings, CutHalfSin, Half2FullFan (:327-380) or Half2Para /
// Fan2Para (:382-470).
//
// TEST INFRASTRUCTURE ONLY: generates the rsq golden fixtures
// (tests/golden/make_rsq_golden.py).  Built by oracle/ref_build.py with g++
// from the reference's source where it lies; nothing of the product links it.
#include "rsq_load.h"

extern "C" int tkref_rsq(const char *path, unsigned first, unsigned last, unsigned axis_move, double distance,
                         double delta_fi, int complete, int parallel, int flip, int invert, double *out,
                         unsigned *w_out, unsigned *h_out)
{
    rsq r{std::string(path)};
    r.SetAxisMove(axis_move);
    r.SetDistance(distance);
    r.SetDeltaFi(delta_fi);
    r.SetCompleting(complete != 0);
    r.SetParallel(parallel != 0);
    r.SetFlip(flip != 0);
    r.SetInvert(invert != 0);
    if (r.LoadImages(first, last) != 0) return -1;
    unsigned sx = 0, sy = 0;
    r.GetSize(sx, sy);
    if (w_out) *w_out = sx;
    if (h_out) *h_out = sy;
    if (!out) return 0;
    return r.ProccessAndCopy(out);
}
