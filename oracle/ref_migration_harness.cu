// Test infrastructure: calls the reference's own Migration::set_wavelet
// (src/migration/migration.cu:54-71), compiled from the reference sources by
// oracle/build_ref.py. FFTW is not installed: the FFTW functions that
// migration.cu names (only its convolution methods call them, never run here)
// are defined below as empty stand-ins so the library links.
#include "migration.cuh"

void* fftw_malloc(size_t) { return nullptr; }
fftw_plan fftw_plan_dft_r2c_1d(int, double*, fftw_complex*, unsigned) { return nullptr; }
fftw_plan fftw_plan_dft_c2r_1d(int, fftw_complex*, double*, unsigned) { return nullptr; }
void fftw_execute(const fftw_plan) {}

namespace {
class Probe : public Migration {
public:
    void set_migration() override {}
    void perform_forward() override {}
    void perform_adjoint() override {}
    void kirchhoff_depth_migration() override {}
    void export_outputs() override {}
    int wavelet_of(float f, float step, float* out, int wmax)
    {
        fmax = f;
        dt = step;
        set_wavelet();
        if (nw > wmax) return -nw;
        for (int k = 0; k < nw; k++) out[k] = wavelet[k];
        delete[] wavelet;
        return nw;
    }
};
}  // namespace

// The reference's Ricker wavelet for max_frequency f and time_spacing dt;
// returns its length (negative when it exceeds wmax).
extern "C" int ref_set_wavelet(float f, float dt, float* out, int wmax)
{
    Probe m;
    return m.wavelet_of(f, dt, out, wmax);
}
