// migration.exe parameters.txt -- the reference's Kirchhoff depth migrations
// (src/migration_main.cpp, mig_type 0-3) on the GB300 engine. The source and
// receiver traveltime tables come from batched solves and stay on the device
// (the reference writes them to eikonal_{src,rec}_<k>.bin and reads them back
// per trace), every trace is cross-correlated with the reference's wavelet
// (sf_adjoint_convolution) and all traces are migrated in one launch.
//   mig_type 0 (IDKDM, KDM.cu:3-55): the image (sf_kirchhoff_image,
//     bit-identical to the reference's launch-per-trace kernel), written to
//     <mig_seismic_folder>IDKDM_result_<nz>x<nx>.bin;
//   mig_type 1 (ADKDM, ADKDM.cu:3-20): angle gathers
//     (sf_kirchhoff_angle_gathers), ADKDM_result_<nz>x<nCMP>x<nang>.bin;
//   mig_type 2, 3 (IDLSKDM, ADLSKDM: LSKDM.cu:3-245): the least-squares
//     loop with the forward operators (sf_kirchhoff_image_forward /
//     sf_kirchhoff_angle_forward + sf_forward_convolution) applied to all
//     traces per call, written to <...>LSKDM_result_..._iteration_<n>.bin with
//     the residual norms in <mig_residuo_folder><type>_convergence_<n>_
//     iterations.txt.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <fstream>
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

// LSKDM (LSKDM.cu:3-235): conjugate-gradient least squares on the host
// vectors, as the reference runs it, with the operators applied to all traces
// per call on the device. The forward operator is demigration then wavelet
// convolution, its adjoint wavelet correlation then migration; traces beyond
// max_offset take no part. FP32 throughout, sums in the reference's order.
struct LsProblem {
    Modeling* m;
    bool angle;
    const float *d_Ts, *d_Tr;
    int ns, nr, nt;
    float dt, fmax, aperture, max_offset, max_angle, da;
    size_t nmodel;
};

static void ls_forward(const LsProblem& P, const float* d_model, float* d_a, float* d_b, float* host_out)
{
    sf_ctx* e = P.m->engine();
    const float* xs = P.m->geometry->xsrc;
    const float* xr = P.m->geometry->xrec;
    if (P.angle)
        sf_check(sf_kirchhoff_angle_forward(e, P.d_Ts, P.d_Tr, P.ns, P.nr, xs, xr, d_model, SF_MEM_DEVICE, P.nt, P.dt,
                                            P.aperture, P.max_offset, P.max_angle, P.da, d_a, SF_MEM_DEVICE, nullptr),
                 e, "sf_kirchhoff_angle_forward");
    else
        sf_check(sf_kirchhoff_image_forward(e, P.d_Ts, P.d_Tr, P.ns, P.nr, xs, xr, d_model, SF_MEM_DEVICE, P.nt, P.dt,
                                            P.aperture, P.max_offset, d_a, SF_MEM_DEVICE, nullptr),
                 e, "sf_kirchhoff_image_forward");
    sf_check(sf_forward_convolution(e, d_a, d_b, P.ns * P.nr, P.nt, P.dt, P.fmax, SF_MEM_DEVICE, nullptr), e,
             "sf_forward_convolution");
    if (cudaMemcpy(host_out, d_b, sizeof(float) * (size_t)P.ns * P.nr * P.nt, cudaMemcpyDeviceToHost) != cudaSuccess)
        throw std::runtime_error("cannot read the modelled traces");
}

static void ls_adjoint(const LsProblem& P, const float* host_res, float* d_a, float* d_b, float* d_model,
                       float* host_out)
{
    sf_ctx* e = P.m->engine();
    const float* xs = P.m->geometry->xsrc;
    const float* xr = P.m->geometry->xrec;
    const size_t nd = (size_t)P.ns * P.nr * P.nt;
    if (cudaMemcpy(d_a, host_res, sizeof(float) * nd, cudaMemcpyHostToDevice) != cudaSuccess)
        throw std::runtime_error("cannot copy the residuals");
    sf_check(sf_adjoint_convolution(e, d_a, d_b, P.ns * P.nr, P.nt, P.dt, P.fmax, SF_MEM_DEVICE, nullptr), e,
             "sf_adjoint_convolution");
    if (P.angle)
        sf_check(sf_kirchhoff_angle_gathers(e, P.d_Ts, P.d_Tr, P.ns, P.nr, xs, xr, d_b, SF_MEM_DEVICE, P.nt, P.dt,
                                            P.aperture, P.max_offset, P.max_angle, P.da, d_model, SF_MEM_DEVICE,
                                            nullptr, nullptr, nullptr),
                 e, "sf_kirchhoff_angle_gathers");
    else
        sf_check(sf_kirchhoff_image(e, P.d_Ts, P.d_Tr, P.ns, P.nr, xs, xr, d_b, SF_MEM_DEVICE, P.nt, P.dt, P.aperture,
                                    P.max_offset, d_model, SF_MEM_DEVICE, nullptr),
                 e, "sf_kirchhoff_image");
    if (cudaMemcpy(host_out, d_model, sizeof(float) * P.nmodel, cudaMemcpyDeviceToHost) != cudaSuccess)
        throw std::runtime_error("cannot read the gradient");
}

static std::vector<float> least_squares(const LsProblem& P, const std::vector<float>& seismic, int max_it,
                                        float smooth, int nang, std::vector<float>& residuo)
{
    const float EPS = 1e-6f;  // migration.cuh:7
    const size_t nd = (size_t)P.ns * P.nr * P.nt, nm = P.nmodel;
    const int nz = P.m->nz;
    const float* xs = P.m->geometry->xsrc;
    const float* xr = P.m->geometry->xrec;
    float *d_a = nullptr, *d_b = nullptr, *d_m = nullptr;
    if (cudaMalloc((void**)&d_a, sizeof(float) * nd) != cudaSuccess ||
        cudaMalloc((void**)&d_b, sizeof(float) * nd) != cudaSuccess ||
        cudaMalloc((void**)&d_m, sizeof(float) * nm) != cudaSuccess)
        throw std::runtime_error("cannot allocate the least-squares buffers");
    std::vector<float> model(nm, 0.0f), gradient(nm), direction(nm, 0.0f), gradient_old(nm, 0.0f);
    std::vector<float> traces(nd), res(nd);
    int iteration = 0;
    while (true) {
        // compute_gradient (LSKDM.cu:46-121)
        cudaMemcpy(d_m, model.data(), sizeof(float) * nm, cudaMemcpyHostToDevice);
        ls_forward(P, d_m, d_a, d_b, traces.data());
        float residuals = 0.0f;
        std::fill(res.begin(), res.end(), 0.0f);
        for (int s = 0; s < P.ns; s++)
            for (int r = 0; r < P.nr; r++) {
                if (!(fabsf(xs[s] - xr[r]) < P.max_offset)) continue;
                const size_t o = ((size_t)s * P.nr + r) * P.nt;
                for (int t = 0; t < P.nt; t++) {
                    const float dobs = seismic[o + t];
                    const float v = (fabsf(dobs) > EPS) ? dobs - traces[o + t] : 0.0f;
                    res[o + t] = v;
                    residuals += v * v;
                }
            }
        ls_adjoint(P, res.data(), d_a, d_b, d_m, gradient.data());
        // compute_residuals (:123-132)
        ++iteration;
        residuo.push_back(sqrtf(residuals));
        if (iteration > max_it) break;
        // compute_direction (:134-161)
        float beta_num = 0.0f, beta_den = 0.0f, alpha_num = 0.0f;
        for (size_t k = 0; k < nm; k++) {
            beta_num += gradient[k] * gradient[k];
            beta_den += gradient_old[k] * gradient_old[k];
        }
        const float beta = beta_num / (beta_den + EPS);
        for (size_t k = 0; k < nm; k++) {
            direction[k] = gradient[k] + beta * direction[k];
            alpha_num += gradient[k] * direction[k];
            gradient_old[k] = gradient[k];
        }
        // compute_stepLength (:163-204)
        cudaMemcpy(d_m, direction.data(), sizeof(float) * nm, cudaMemcpyHostToDevice);
        ls_forward(P, d_m, d_a, d_b, traces.data());
        float alpha_den = 0.0f;
        for (int s = 0; s < P.ns; s++)
            for (int r = 0; r < P.nr; r++) {
                if (!(fabsf(xs[s] - xr[r]) < P.max_offset)) continue;
                const size_t o = ((size_t)s * P.nr + r) * P.nt;
                for (int t = 0; t < P.nt; t++) alpha_den += traces[o + t] * traces[o + t];
            }
        const float alpha = alpha_num / (alpha_den + EPS);
        // regularization: none in the image domain (IDLSKDM.cu:12-17); second
        // difference along angle, mirrored at both ends, in the angle domain
        // (ADLSKDM.cu:12-41). A single angle bin has no neighbour: skipped.
        if (P.angle && nang > 1) {
            const size_t ncmp = nm / ((size_t)nz * nang);
            for (size_t c = 0; c < ncmp; c++)
                for (int z = 0; z < nz; z++)
                    for (int a = 0; a < nang; a++) {
                        const size_t tg = z + (size_t)a * nz + c * nang * nz;
                        const size_t fw = z + (size_t)(a + 1) * nz + c * nang * nz;
                        const size_t bw = z + (size_t)(a - 1) * nz + c * nang * nz;
                        const size_t l = (a == 0) ? fw : bw, h = (a == nang - 1) ? bw : fw;
                        direction[tg] += smooth * (model[h] - 2.0f * model[tg] + model[l]) / (P.da * P.da);
                    }
        }
        // update_model (:206-210)
        for (size_t k = 0; k < nm; k++) model[k] = model[k] + alpha * direction[k];
    }
    cudaFree(d_a);
    cudaFree(d_b);
    cudaFree(d_m);
    return model;
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
        if (mig_type < 0 || mig_type > 3) throw std::invalid_argument("mig_type must be 0, 1, 2 or 3");
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
        std::string out_path;
        std::vector<float> out;
        const bool angle = (mig_type == 1 || mig_type == 3);
        float max_angle = 0.0f, da = 1.0f;
        int nang = 0, ncmp = 0;
        if (angle) {
            max_angle = std::stof(catch_parameter("mig_max_angle", file));
            da = std::stof(catch_parameter("mig_angle_spacing", file));
            sf_check(sf_kirchhoff_angle_gathers(m->engine(), d_Ts, d_Tr, ns, nr, m->geometry->xsrc, m->geometry->xrec,
                                                nullptr, SF_MEM_HOST, nt, dt, aperture, max_offset, max_angle, da,
                                                nullptr, SF_MEM_HOST, &nang, &ncmp, nullptr),
                     m->engine(), "sf_kirchhoff_angle_gathers");
        }
        const std::string dims = angle ? std::to_string(m->nz) + "x" + std::to_string(ncmp) + "x" + std::to_string(nang)
                                       : std::to_string(m->nz) + "x" + std::to_string(m->nx);
        const size_t nmodel = angle ? (size_t)m->nz * nang * ncmp : (size_t)m->nPoints;
        out.resize(nmodel);
        if (mig_type <= 1) {
            sf_check(sf_adjoint_convolution(m->engine(), data.data(), corr.data(), ns * nr, nt, dt, fmax,
                                            SF_MEM_HOST, nullptr),
                     m->engine(), "sf_adjoint_convolution");
            if (angle)
                sf_check(sf_kirchhoff_angle_gathers(m->engine(), d_Ts, d_Tr, ns, nr, m->geometry->xsrc,
                                                    m->geometry->xrec, corr.data(), SF_MEM_HOST, nt, dt, aperture,
                                                    max_offset, max_angle, da, out.data(), SF_MEM_HOST, nullptr,
                                                    nullptr, nullptr),
                         m->engine(), "sf_kirchhoff_angle_gathers");
            else
                sf_check(sf_kirchhoff_image(m->engine(), d_Ts, d_Tr, ns, nr, m->geometry->xsrc, m->geometry->xrec,
                                            corr.data(), SF_MEM_HOST, nt, dt, aperture, max_offset, out.data(),
                                            SF_MEM_HOST, nullptr),
                         m->engine(), "sf_kirchhoff_image");
            out_path = seismic_folder + (angle ? "ADKDM" : "IDKDM") + "_result_" + dims + ".bin";
        } else {
            // LSKDM::initialization and Migration::set_parameters (LSKDM.cu:31-44,
            // migration.cu:9-10)
            const int max_it = std::stoi(catch_parameter("mig_max_iteration", file));
            const std::string residuo_folder = catch_parameter("mig_residuo_folder", file);
            const float smooth = std::stof(catch_parameter("mig_smooth_lambda", file));
            const std::string type = angle ? "ADLSKDM" : "IDLSKDM";
            LsProblem P{m, angle, d_Ts, d_Tr, ns, nr, nt, dt, fmax, aperture, max_offset, max_angle, da, nmodel};
            std::vector<float> residuo;
            out = least_squares(P, data, max_it, smooth, nang, residuo);
            // LSKDM::export_outputs (LSKDM.cu:229-245)
            const std::string rpath = residuo_folder + type + "_convergence_" + std::to_string(max_it) + "_iterations.txt";
            std::ofstream rf(rpath, std::ios::out);
            for (float v : residuo) rf << v << "\n";
            out_path = seismic_folder + type + "_result_" + dims + "_iteration_" + std::to_string(max_it) + ".bin";
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
