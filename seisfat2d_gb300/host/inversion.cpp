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
    // the reference parses the filter width with stoi (inversion.cpp:13): "5.0" -> 5
    smoother_stdv = (float)std::stoi(param_or("gaussian_filter_stdv", parameters, "5"));
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
    sf_check(sf_batch_forward(modeling->engine(), modeling->anisotropic(), shots.data(), ns, modeling->geometry->xrec,
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

double Inversion::misfit_of_current()
{
    const int ns = modeling->geometry->nsrc, nr = modeling->geometry->nrec;
    std::vector<sf_shot> shots(ns);
    for (int s = 0; s < ns; s++) shots[s] = {modeling->geometry->xsrc[s], modeling->geometry->zsrc[s], 0, 0};
    std::vector<float> pk((size_t)ns * nr);
    sf_check(sf_batch_forward(modeling->engine(), modeling->anisotropic(), shots.data(), ns, modeling->geometry->xrec,
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
// the largest model cell by 1% of the mean slowness. Each trial update
// (scale, smoothing of model_smoothing, S += dS on the interior) runs on the
// device (sf_update_slowness) from the current model; the accepted one is
// left in dS and in the engine.
void Inversion::optimization()
{
    Modeling* m = modeling;
    sf_check(sf_batch_misfit_gradient(m->engine(), dobs, SF_MEM_HOST, &misfit, grad, SF_MEM_HOST, nullptr),
             m->engine(), "sf_batch_misfit_gradient");
    double gmax = 0.0, smean = 0.0;
    for (int index = 0; index < n_model; index++) {
        int i = index % m->nz, j = index / m->nz;
        gmax = std::max(gmax, (double)std::fabs(grad[(i + m->nb) + (j + m->nb) * m->nzz]));
        smean += m->S[(i + m->nb) + (j + m->nb) * m->nzz];
    }
    smean /= n_model;
    std::fill(dS, dS + n_model, 0.0f);
    if (gmax == 0.0) return;
    double alpha = 0.01 * smean / gmax;
    const int samples = smooth_model_per_iteration ? smoother_samples : 0;
    for (int tries = 0; tries < 8; tries++, alpha *= 0.5) {
        sf_check(sf_set_slowness(m->engine(), m->S, SF_LAYOUT_PADDED, SF_MEM_HOST), m->engine(), "sf_set_slowness");
        sf_check(sf_update_slowness(m->engine(), grad, SF_MEM_HOST, (float)-alpha, smoother_stdv, samples, dS,
                                    SF_MEM_HOST, nullptr),
                 m->engine(), "sf_update_slowness");
        if (misfit_of_current() < misfit) return;
    }
    std::fill(dS, dS + n_model, 0.0f);  // no trial lowered the misfit
    sf_check(sf_set_slowness(m->engine(), m->S, SF_LAYOUT_PADDED, SF_MEM_HOST), m->engine(), "sf_set_slowness");
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

// tomography_iso.cpp:77-92 (dS was smoothed and applied on the device by the
// line search; the host copy of S follows with the same FP32 sums)
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

// ------------------------------------------------------------ Tomography_VTI

void Tomography_VTI::set_modeling_type()
{
    eikonal = new Eikonal_ANI();
    modeling = eikonal;
    modeling->parameters = parameters;
    modeling->set_parameters();
    inversion_name = "tomography_vti";
    inversion_method = "Anisotropic First-Arrival Tomography";
    E.assign(modeling->nPoints, 0.0f);
    D.assign(modeling->nPoints, 0.0f);
    dE.assign(modeling->nPoints, 0.0f);
    dD.assign(modeling->nPoints, 0.0f);
    eikonal->get_stiffness_VTI(E.data(), D.data());
}

// Steepest descent on J in (S, epsilon, delta): the first trial moves the
// largest cell of each parameter by 1% of the mean slowness, 0.01 in epsilon,
// 0.01 in delta; each trial halves all three. Every trial update is smoothed
// (sf_update_slowness for S, sf_smooth_model for epsilon and delta), applied
// to the engine's model and stiffness, and kept when the misfit falls.
void Tomography_VTI::optimization()
{
    Modeling* m = modeling;
    sf_ctx* e = m->engine();
    const int nP = m->nPoints;
    std::vector<float> g11(m->matsize), g13(m->matsize);
    sf_check(sf_batch_misfit_gradient(e, dobs, SF_MEM_HOST, &misfit, grad, SF_MEM_HOST, nullptr), e,
             "sf_batch_misfit_gradient");
    sf_check(sf_batch_stiffness_gradient(e, g11.data(), g13.data(), SF_MEM_HOST, nullptr), e,
             "sf_batch_stiffness_gradient");
    std::vector<float> gE(nP), gD(nP);
    double gmaxS = 0.0, gmaxE = 0.0, gmaxD = 0.0, smean = 0.0;
    const std::vector<float>& C13 = eikonal->stiffness(1);
    const std::vector<float>& C33 = eikonal->stiffness(3);
    const std::vector<float>& C55 = eikonal->stiffness(5);
    for (int index = 0; index < nP; index++) {
        const int i = index % m->nz + m->nb, j = index / m->nz + m->nb;
        const size_t k = (size_t)i + (size_t)j * m->nzz;
        const double c13 = C13[k], c33 = C33[k], c55 = C55[k];
        gE[index] = (float)((double)g11[k] * 2.0 * c33);
        gD[index] = (float)((double)g13[k] * c33 * (c33 - c55) / (c13 + c55));
        gmaxS = std::max(gmaxS, (double)std::fabs(grad[k]));
        gmaxE = std::max(gmaxE, (double)std::fabs(gE[index]));
        gmaxD = std::max(gmaxD, (double)std::fabs(gD[index]));
        smean += m->S[k];
    }
    smean /= nP;
    std::fill(dS, dS + nP, 0.0f);
    std::fill(dE.begin(), dE.end(), 0.0f);
    std::fill(dD.begin(), dD.end(), 0.0f);
    if (gmaxS == 0.0 && gmaxE == 0.0 && gmaxD == 0.0) return;
    double aS = gmaxS > 0.0 ? 0.01 * smean / gmaxS : 0.0;
    double aE = gmaxE > 0.0 ? 0.01 / gmaxE : 0.0, aD = gmaxD > 0.0 ? 0.01 / gmaxD : 0.0;
    const int samples = smooth_samples();
    std::vector<float> tE(nP), tD(nP), sE(nP), sD(nP);
    for (int tries = 0; tries < 8; tries++, aS *= 0.5, aE *= 0.5, aD *= 0.5) {
        sf_check(sf_set_slowness(e, m->S, SF_LAYOUT_PADDED, SF_MEM_HOST), e, "sf_set_slowness");
        sf_check(sf_update_slowness(e, grad, SF_MEM_HOST, (float)-aS, smooth_stdv(), samples, dS, SF_MEM_HOST,
                                    nullptr),
                 e, "sf_update_slowness");
        for (int index = 0; index < nP; index++) {
            tE[index] = (float)(-aE * gE[index]);
            tD[index] = (float)(-aD * gD[index]);
        }
        if (samples > 0) {
            sf_check(sf_smooth_model(e, tE.data(), sE.data(), smooth_stdv(), samples, SF_MEM_HOST, nullptr), e,
                     "sf_smooth_model");
            sf_check(sf_smooth_model(e, tD.data(), sD.data(), smooth_stdv(), samples, SF_MEM_HOST, nullptr), e,
                     "sf_smooth_model");
        } else {
            sE = tE;
            sD = tD;
        }
        std::vector<float> nE(nP), nD(nP);
        for (int index = 0; index < nP; index++) {
            nE[index] = E[index] + sE[index];
            nD[index] = D[index] + sD[index];
        }
        eikonal->set_stiffness_VTI(nE.data(), nD.data());
        if (misfit_of_current() < misfit) {
            dE = sE;
            dD = sD;
            return;
        }
    }
    // no trial lowered the misfit: the model stays
    std::fill(dS, dS + nP, 0.0f);
    sf_check(sf_set_slowness(e, m->S, SF_LAYOUT_PADDED, SF_MEM_HOST), e, "sf_set_slowness");
    eikonal->set_stiffness_VTI(E.data(), D.data());
}

// tomography_vti.cpp:121-139: S += dS on the interior, E += dE, D += dD, the
// stiffness rebuilt (the accepted trial already left all three in the engine)
void Tomography_VTI::model_update()
{
    for (int index = 0; index < modeling->nPoints; index++) {
        int i = index % modeling->nz, j = index / modeling->nz;
        modeling->S[(i + modeling->nb) + (j + modeling->nb) * modeling->nzz] += dS[index];
        E[index] += dE[index];
        D[index] += dD[index];
    }
    modeling->copy_slowness_to_device();
    eikonal->set_stiffness_VTI(E.data(), D.data());
}

void Tomography_VTI::export_estimated_models()
{
    std::vector<float> vp(modeling->nPoints);
    modeling->reduce_boundary(modeling->S, vp.data());
    for (auto& v : vp) v = 1.0f / v;
    const std::string dims = std::to_string(modeling->nz) + "x" + std::to_string(modeling->nx) + ".bin";
    export_binary_float(estimated_model_folder + inversion_name + "_final_model_vp_" + dims, vp.data(),
                        modeling->nPoints);
    export_binary_float(estimated_model_folder + inversion_name + "_final_model_ep_" + dims, E.data(),
                        modeling->nPoints);
    export_binary_float(estimated_model_folder + inversion_name + "_final_model_dl_" + dims, D.data(),
                        modeling->nPoints);
}
