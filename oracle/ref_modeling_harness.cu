// Test infrastructure: calls the reference's own host-side setup methods,
// Modeling::expand_boundary (src/modeling/modeling.cu:204-232) and
// Modeling::compression (modeling.cu:264-279), compiled from the reference
// sources by oracle/build_ref.py (single-threaded, so compression's min/max
// loop is the serial one). Used only by tests to pin the oracle's padding and
// Cij quantisation.
#include "modeling.cuh"

namespace {
class Probe : public Modeling {
public:
    void set_conditions() override {}
    void time_propagation() override {}
    void quantise(float* in, uintc* out, int n, float& mx, float& mn) { compression(in, out, n, mx, mn); }
};
}  // namespace

// in: nz x nx (z fastest); out: (nz + 2 nb) x (nx + 2 nb)
extern "C" void ref_expand_boundary(float* in, float* out, int nx, int nz, int nb)
{
    Probe m;
    m.nx = nx;
    m.nz = nz;
    m.nb = nb;
    m.nPoints = nx * nz;
    m.nxx = nx + 2 * nb;
    m.nzz = nz + 2 * nb;
    m.matsize = m.nxx * m.nzz;
    m.expand_boundary(in, out);
}

extern "C" void ref_compression(float* in, unsigned short* out, int n, float* vmax, float* vmin)
{
    Probe m;
    m.quantise(in, out, n, *vmax, *vmin);
}
