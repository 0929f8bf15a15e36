#include "inversion.hpp"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <iostream>
#include <stdexcept>

#include "admin.hpp"

static std::string param_or(const std::string& key, const std::string& file, const std::string& dflt)
{
    std::string v = catch_parameter(key, file);
    return v.empty() ? dflt : v;
}

void Inversion::set_parameters()
{
    max_iteration = std::stoi(param_or("inv_max_it", parameters, "5"));
    obs_data_folder = catch_parameter("inv_data_folder", parameters);
    obs_data_prefix = catch_parameter("inv_data_prefix", parameters);
    smoother_stdv = std::stof(param_or("gaussian_filter_stdv", parameters, "5.0"));
    smoother_samples = std::stoi(param_or("gaussian_filter_samples", parameters, "11"));
    convergence_map_folder = catch_parameter("inv_residuo_folder", parameters);
    estimated_model_folder = catch_parameter("inv_output_folder", parameters);
    smooth_model_per_iteration = str2bool(param_or("smooth_per_iteration", parameters, "true"));
    set_modeling_type();
}

void Inversion::import_obsData()
{
    const int ns = modeling->geometry->nsrc, nr = modeling->geometry->nrec;
    n_data = ns * nr;
    n_model = modeling->nPoints;
    delete[] dcal; delete[] dobs;
    dcal = new float[n_data]();
    dobs = new float[n_data]();
    for (int s = 0; s < ns; s++) {
        std::string path = obs_data_folder + obs_data_prefix + std::to_string(s + 1) + ".bin";
        import_binary_float(path, dobs + (size_t)s * nr, nr);
    }
    delete[] grad;
    grad = new float[modeling->matsize]();
    delete[] dS;
    dS = new float[n_model]();
}

void Inversion::show_information()
{
    std::cout << inversion_method << ": ";
    if (iteration == max_iteration) std::cout << "checking final residuo\n";
    else {
        std::cout << "iteration " << iteration + 1 << " of " << max_iteration;
        if (!residuo.empty()) std::cout << ", previous residuo " << residuo.back();
        std::cout << "\n";
    }
}

void Inversion::forward_modeling()
{
    show_information();
    const int ns = modeling->geometry->nsrc, nr = modeling->geometry->nrec;
    std::vector<sf_shot> shots(ns);
    for (int s = 0; s < ns; s++) shots[s] = {modeling->geometry->xsrc[s], modeling->geometry->zsrc[s], 0, 0};
    sf_check(sf_batch_forward(modeling->engine(), 0, shots.data(), ns, modeling->geometry->xrec,
                              modeling->geometry->zrec, nr, dcal, SF_MEM_HOST, SF_KEEP_TAPE, nullptr),
             modeling->engine(), "sf_batch_forward");
}

void Inversion::check_convergence()
{
    double sq = 0.0;
    for (int i = 0; i < n_data; i++) {
        double r = (double)dobs[i] - (double)dcal[i];
        if (r == r) sq += r * r;
    }
    residuo.push_back((float)std::sqrt(sq));
    if (iteration >= max_iteration) {
        std::cout << "Final residuo: " << residuo.back() << "\n";
        converged = true;
    } else {
        iteration += 1;
        converged = false;
    }
}

double Inversion::misfit_of(const float* S_padded)
{
    const int ns = modeling->geometry->nsrc, nr = modeling->geometry->nrec;
    sf_check(sf_set_slowness(modeling->engine(), S_padded, SF_LAYOUT_PADDED, SF_MEM_HOST), modeling->engine(),
             "sf_set_slowness");
    std::vector<sf_shot> shots(ns);
    for (int s = 0; s < ns; s++) shots[s] = {modeling->geometry->xsrc[s], modeling->geometry->zsrc[s], 0, 0};
    std::vector<float> pk((size_t)ns * nr);
    sf_check(sf_batch_forward(modeling->engine(), 0, shots.data(), ns, modeling->geometry->xrec,
                              modeling->geometry->zrec, nr, pk.data(), SF_MEM_HOST, 0, nullptr),
             modeling->engine(), "sf_batch_forward");
    double J = 0.0;
    for (size_t i = 0; i < pk.size(); i++) {
        double r = (double)pk[i] - (double)dobs[i];
        if (r == r) J += 0.5 * r * r;
    }
    return J;
}

// Steepest descent on J = 1/2 |picks - dobs|^2: the adjoint-state gradient of
// the taped forward, then a backtracking line search whose first step moves
// the largest model cell by 1% of the mean slowness.
void Inversion::optimization()
{
    Modeling* m = modeling;
    sf_check(sf_batch_misfit_gradient(m->engine(), dobs, SF_MEM_HOST, &misfit, grad, SF_MEM_HOST, nullptr),
             m->engine(), "sf_batch_misfit_gradient");
    std::vector<float> g(n_model);
    double gmax = 0.0, smean = 0.0;
    for (int index = 0; index < n_model; index++) {
        int i = index % m->nz, j = index / m->nz;
        g[index] = grad[(i + m->nb) + (j + m->nb) * m->nzz];
        gmax = std::max(gmax, (double)std::fabs(g[index]));
        smean += m->S[(i + m->nb) + (j + m->nb) * m->nzz];
    }
    smean /= n_model;
    std::fill(dS, dS + n_model, 0.0f);
    if (gmax == 0.0) return;
    double alpha = 0.01 * smean / gmax;
    std::vector<float> trial(m->S, m->S + m->matsize);
    for (int tries = 0; tries < 8; tries++, alpha *= 0.5) {
        for (int index = 0; index < n_model; index++) dS[index] = (float)(-alpha * g[index]);
        if (smooth_model_per_iteration) model_smoothing(dS);
        std::copy(m->S, m->S + m->matsize, trial.begin());
        for (int index = 0; index < n_model; index++) {
            int i = index % m->nz, j = index / m->nz;
            trial[(i + m->nb) + (j + m->nb) * m->nzz] += dS[index];
        }
        if (misfit_of(trial.data()) < misfit) break;
        if (tries == 7) std::fill(dS, dS + n_model, 0.0f);
    }
    sf_check(sf_set_slowness(m->engine(), m->S, SF_LAYOUT_PADDED, SF_MEM_HOST), m->engine(), "sf_set_slowness");
}

// inversion.cpp:347-383
void Inversion::model_smoothing(float* model)
{
    const int nx = modeling->nx, nz = modeling->nz;
    const int aux_nx = nx + 2 * smoother_samples, aux_nz = nz + 2 * smoother_samples;
    std::vector<float> dm_aux((size_t)aux_nx * aux_nz, 0.0f), dm_smooth((size_t)aux_nx * aux_nz, 0.0f);
    for (int index = 0; index < nx * nz; index++) {
        int i = index % nz, j = index / nz;
        dm_aux[(i + smoother_samples) + (size_t)(j + smoother_samples) * aux_nz] = model[i + j * nz];
    }
    smooth_matrix(dm_aux.data(), dm_smooth.data(), aux_nx, aux_nz);
    for (int index = 0; index < nx * nz; index++) {
        int i = index % nz, j = index / nz;
        model[i + j * nz] = dm_smooth[(i + smoother_samples) + (size_t)(j + smoother_samples) * aux_nz];
    }
}

// inversion.cpp:385-447: normalised Gaussian 1/(pi s) exp(-r^2 / 2s^2)
void Inversion::smooth_matrix(float* input, float* output, int nx, int nz)
{
    const int n = smoother_samples;
    std::vector<float> kernel((size_t)n * n, 0.0f);
    std::copy(input, input + (size_t)nx * nz, output);
    const int mid = n / 2;
    kernel[mid + mid * n] = 1.0f;
    if (smoother_stdv != 0.0f) {
        float sum = 0.0f;
        for (int x = -mid; x <= mid; x++)
            for (int z = -mid; z <= mid; z++) {
                int index = (z + mid) + (x + mid) * n;
                float r = std::sqrt((float)(x * x + z * z));
                kernel[index] = 1.0f / ((float)M_PI * smoother_stdv) *
                                std::exp(-((r * r) / (2.0f * smoother_stdv * smoother_stdv)));
                sum += kernel[index];
            }
        for (auto& k : kernel) k /= sum;
    }
    for (int j = mid; j < nx - mid; j++)
        for (int i = mid; i < nz - mid; i++) {
            float accum = 0.0f;
            for (int xk = 0; xk < n; xk++)
                for (int zk = 0; zk < n; zk++)
                    accum += input[(i - mid + zk) + (size_t)(j - mid + xk) * nz] * kernel[zk + xk * n];
            output[i + (size_t)j * nz] = accum;
        }
}

void Inversion::export_results()
{
    export_estimated_models();
    std::string path = convergence_map_folder + inversion_name + "_convergence_" + std::to_string(iteration) +
                       "_iterations.txt";
    std::ofstream res(path, std::ios::out);
    for (float r : residuo) res << r << "\n";
}

Inversion::~Inversion()
{
    delete[] dcal;
    delete[] dobs;
    delete[] dS;
    delete[] grad;
    delete modeling;
}

// ------------------------------------------------------------ Tomography_ISO

void Tomography_ISO::set_modeling_type()
{
    modeling = new Eikonal_ISO();
    modeling->parameters = parameters;
    modeling->set_parameters();
    inversion_name = "tomography_iso";
    inversion_method = "Isotropic First-Arrival Tomography";
}

// tomography_iso.cpp:77-92 (dS is already smoothed by the line search)
void Tomography_ISO::model_update()
{
    for (int index = 0; index < modeling->nPoints; index++) {
        int i = index % modeling->nz, j = index / modeling->nz;
        modeling->S[(i + modeling->nb) + (j + modeling->nb) * modeling->nzz] += dS[index];
    }
    modeling->copy_slowness_to_device();
}

void Tomography_ISO::export_estimated_models()
{
    std::vector<float> vp(modeling->nPoints);
    modeling->reduce_boundary(modeling->S, vp.data());
    for (auto& v : vp) v = 1.0f / v;
    std::string path = estimated_model_folder + inversion_name + "_final_model_vp_" + std::to_string(modeling->nz) +
                       "x" + std::to_string(modeling->nx) + ".bin";
    export_binary_float(path, vp.data(), modeling->nPoints);
}
