// Test infrastructure: calls the reference's own smoothing methods,
// Inversion::model_smoothing and Inversion::smooth_matrix
// (src/inversion/inversion.cpp:347-447), compiled from the reference source
// by oracle/build_ref.py with the declarations of its force-included shim
// header. Used only by tests to pin the oracle's smoothing restatement.

// model: nz x nx floats (z fastest), smoothed in place exactly as
// Tomography_ISO::model_update smooths dS (gaussian_filter_samples = samples,
// gaussian_filter_stdv = stdv).
extern "C" void ref_model_smoothing(float* model, int nx, int nz, int samples, float stdv)
{
    Geometry g;
    Modeling m;
    m.nx = nx;
    m.nz = nz;
    m.nPoints = nx * nz;
    m.geometry = &g;
    Inversion inv;
    inv.modeling = &m;
    inv.smoother_samples = samples;
    inv.smoother_stdv = stdv;
    inv.smooth_model_per_iteration = true;
    inv.model_smoothing(model);
}
