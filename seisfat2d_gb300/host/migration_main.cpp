// migration.exe parameters.txt -- the reference's image-domain Kirchhoff depth
// migration (src/migration_main.cpp with mig_type = 0, IDKDM; KDM.cu:3-55) on
// the GB300 engine. The source and receiver traveltime tables come from
// batched solves and stay on the device (the reference writes them to
// eikonal_{src,rec}_<k>.bin and reads them back per trace), every trace is
// cross-correlated with the reference's wavelet (sf_adjoint_convolution) and
// the image is summed over all traces in one launch (sf_kirchhoff_image,
// bit-identical to the reference's launch-per-trace kernel on the same
// tables and traces). mig_type = 0 writes the image
// <mig_seismic_folder>IDKDM_result_<nz>x<nx>.bin; mig_type = 1 (ADKDM,
// ADKDM.cu:3-20) writes angle gathers <mig_seismic_folder>ADKDM_result_
// <nz>x<nCMP>x<nang>.bin (sf_kirchhoff_angle_gathers). The least-squares
// variants (mig_type 2, 3) are not built.
#include <cuda_runtime.h>

#include <chrono>
#include <iostream>
#include <stdexcept>
#include <vector>

#include "admin.hpp"
#include "modeling.hpp"

static void tables_on_device(Modeling* m, const float* x, const float* z, int n, float* d_tables)
{
    const int chunk = 256;
    for (int first = 0; first < n; first += chunk) {
        const int cnt = std::min(chunk, n - first);
        std::vector<sf_shot> shots(cnt);
        for (int k = 0; k < cnt; k++) shots[k] = {x[first + k], z[first + k], 0, 0};
        sf_check(sf_batch_forward(m->engine(), m->anisotropic(), shots.data(), cnt, nullptr, nullptr, 0, nullptr,
                                  SF_MEM_HOST, SF_KEEP_TABLES, nullptr),
                 m->engine(), "sf_batch_forward");
        for (int k = 0; k < cnt; k++)
            sf_check(sf_batch_table(m->engine(), k, d_tables + (size_t)(first + k) * m->matsize, SF_MEM_DEVICE,
                                    nullptr),
                     m->engine(), "sf_batch_table");
    }
}

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::cerr << "usage: migration.exe parameters.txt\n";
        return 1;
    }
    try {
        const std::string file = argv[1];
        const int mig_type = std::stoi(catch_parameter("mig_type", file));
        if (mig_type != 0 && mig_type != 1)
            throw std::invalid_argument("only mig_type = 0 (image domain) and 1 (angle domain) are built");
        const int nt = std::stoi(catch_parameter("time_samples", file));
        const float dt = std::stof(catch_parameter("time_spacing", file));
        const float fmax = std::stof(catch_parameter("max_frequency", file));
        const float aperture = std::stof(catch_parameter("mig_aperture", file));
        const float max_offset = std::stof(catch_parameter("mig_max_offset", file));
        const std::string data_folder = catch_parameter("mig_data_folder", file);
        const std::string data_prefix = catch_parameter("mig_data_prefix", file);
        const std::string seismic_folder = catch_parameter("mig_seismic_folder", file);
        Modeling* m = str2bool(catch_parameter("anisotropy", file)) ? (Modeling*)new Eikonal_ANI()
                                                                     : (Modeling*)new Eikonal_ISO();
        m->parameters = file;
        m->set_parameters();
        const int ns = m->geometry->nsrc, nr = m->geometry->nrec;
        auto ti = std::chrono::system_clock::now();
        float *d_Ts = nullptr, *d_Tr = nullptr;
        if (cudaMalloc((void**)&d_Ts, sizeof(float) * (size_t)m->matsize * ns) != cudaSuccess ||
            cudaMalloc((void**)&d_Tr, sizeof(float) * (size_t)m->matsize * nr) != cudaSuccess)
            throw std::runtime_error("cannot allocate the traveltime tables on the device");
        tables_on_device(m, m->geometry->xsrc, m->geometry->zsrc, ns, d_Ts);
        tables_on_device(m, m->geometry->xrec, m->geometry->zrec, nr, d_Tr);
        // traces: per source nt x nrec, trace-major (KDM.cu:14-15, :46-47)
        std::vector<float> data((size_t)ns * nr * nt), corr(data.size());
        for (int s = 0; s < ns; s++)
            import_binary_float(data_folder + data_prefix + std::to_string(s + 1) + ".bin",
                                data.data() + (size_t)s * nr * nt, nr * nt);
        sf_check(sf_adjoint_convolution(m->engine(), data.data(), corr.data(), ns * nr, nt, dt, fmax, SF_MEM_HOST,
                                        nullptr),
                 m->engine(), "sf_adjoint_convolution");
        std::string out_path;
        std::vector<float> out;
        if (mig_type == 0) {
            out.resize((size_t)m->nPoints);
            sf_check(sf_kirchhoff_image(m->engine(), d_Ts, d_Tr, ns, nr, m->geometry->xsrc, m->geometry->xrec,
                                        corr.data(), SF_MEM_HOST, nt, dt, aperture, max_offset, out.data(),
                                        SF_MEM_HOST, nullptr),
                     m->engine(), "sf_kirchhoff_image");
            out_path = seismic_folder + "IDKDM_result_" + std::to_string(m->nz) + "x" + std::to_string(m->nx) + ".bin";
        } else {
            const float max_angle = std::stof(catch_parameter("mig_max_angle", file));
            const float da = std::stof(catch_parameter("mig_angle_spacing", file));
            int nang = 0, ncmp = 0;
            sf_check(sf_kirchhoff_angle_gathers(m->engine(), d_Ts, d_Tr, ns, nr, m->geometry->xsrc, m->geometry->xrec,
                                                nullptr, SF_MEM_HOST, nt, dt, aperture, max_offset, max_angle, da,
                                                nullptr, SF_MEM_HOST, &nang, &ncmp, nullptr),
                     m->engine(), "sf_kirchhoff_angle_gathers");
            out.resize((size_t)m->nz * nang * ncmp);
            sf_check(sf_kirchhoff_angle_gathers(m->engine(), d_Ts, d_Tr, ns, nr, m->geometry->xsrc, m->geometry->xrec,
                                                corr.data(), SF_MEM_HOST, nt, dt, aperture, max_offset, max_angle, da,
                                                out.data(), SF_MEM_HOST, nullptr, nullptr, nullptr),
                     m->engine(), "sf_kirchhoff_angle_gathers");
            out_path = seismic_folder + "ADKDM_result_" + std::to_string(m->nz) + "x" + std::to_string(ncmp) + "x" +
                       std::to_string(nang) + ".bin";
        }
        auto tf = std::chrono::system_clock::now();
        export_binary_float(out_path, out.data(), (int)out.size());
        cudaFree(d_Ts);
        cudaFree(d_Tr);
        std::chrono::duration<double> elapsed = tf - ti;
        std::cout << "\nRun time: " << elapsed.count() << " s." << std::endl;
        delete m;
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        return 2;
    }
    return 0;
}
