// Test infrastructure: calls the reference's own host-side methods,
// Modeling::expand_boundary (src/modeling/modeling.cu:204-232),
// Modeling::compression (modeling.cu:264-279) and the receiver rule of
// Modeling::compute_seismogram (modeling.cu:161-194, with cubic2d of
// admin.cpp:121-133), compiled from the reference sources by
// oracle/build_ref.py (single-threaded, so compression's min/max loop is the
// serial one). Used only by tests, on a machine without a GPU, to pin the
// oracle's padding, Cij quantisation and picks.
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

// Picks of the padded field T ((nz + 2 nb) x (nx + 2 nb), z fastest) at the
// receivers, by the reference's compute_seismogram. Its first step copies
// d_T to T with cudaMemcpy; with d_T = T and no GPU that copy fails and
// leaves T as given, so the host loop reads the field passed in.
extern "C" void ref_compute_seismogram(float* T, int nx, int nz, int nb, float dx, float dz, float* rx, float* rz,
                                       int nrec, float* out)
{
    Probe m;
    m.nx = nx;
    m.nz = nz;
    m.nb = nb;
    m.nPoints = nx * nz;
    m.nxx = nx + 2 * nb;
    m.nzz = nz + 2 * nb;
    m.matsize = m.nxx * m.nzz;
    m.dx = dx;
    m.dz = dz;
    m.T = T;
    m.d_T = T;
    Geometry g;
    g.nrec = nrec;
    g.xrec = rx;
    g.zrec = rz;
    m.geometry = &g;
    m.seismogram = out;
    m.compute_seismogram();
}
