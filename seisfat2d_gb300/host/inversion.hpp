// Drop-in for the reference's first-arrival tomography
// (src/inversion/inversion.hpp:7-98, tomography_iso.hpp): same driver shape
// (forward_modeling -> check_convergence -> optimization -> model_update),
// with the gradient/ray-tracing step and the LSCG solve replaced by the
// engine's adjoint-state gradient and a backtracking line search on the FP64
// misfit.
#ifndef SF_HOST_INVERSION_HPP
#define SF_HOST_INVERSION_HPP

#include <string>
#include <vector>

#include "modeling.hpp"

class Inversion
{
private:
    int smoother_samples = 11;
    float smoother_stdv = 5.0f;
    std::string obs_data_folder, obs_data_prefix, convergence_map_folder;
    bool smooth_model_per_iteration = true;
    void show_information();

protected:
    int n_data = 0, n_model = 0;
    int iteration = 0, max_iteration = 0;
    float* dcal = nullptr;
    float* dobs = nullptr;
    float* dS = nullptr;     // model update on the nz x nx model
    float* grad = nullptr;   // dJ/dS on the padded grid
    double misfit = 0.0;
    Modeling* modeling = nullptr;
    std::vector<float> residuo;
    std::string inversion_name, inversion_method, estimated_model_folder;

    virtual void set_modeling_type() = 0;
    virtual void export_estimated_models() = 0;

    double misfit_of_current();  // one forward of the engine's current model, picks only
    int smooth_samples() const { return smooth_model_per_iteration ? smoother_samples : 0; }
    float smooth_stdv() const { return smoother_stdv; }

public:
    bool converged = false;
    std::string parameters;

    void set_parameters();     // inversion.cpp:3-22 (keys as written in run/parameters.txt)
    void import_obsData();     // inversion.cpp:24-50
    void forward_modeling();   // inversion.cpp:52-67: all shots in one taped launch
    void check_convergence();  // inversion.cpp:179-198
    virtual void optimization();  // adjoint gradient + line search (replaces :200-345)
    virtual void model_update() = 0;
    void export_results();     // inversion.cpp:449-463
    virtual ~Inversion();
};

class Tomography_ISO : public Inversion
{
private:
    void set_modeling_type() override;        // tomography_iso.cpp:3-13
    void export_estimated_models() override;  // tomography_iso.cpp:94-104

public:
    void model_update() override;  // tomography_iso.cpp:77-92
};

// Anisotropic (VTI) first-arrival tomography (the reference's
// Tomography_VTI, tomography_vti.cpp:3-168, which does not build: it calls
// Eikonal_ANI::get/set_stiffness_VTI, never defined, and its E and D blocks
// have zero right-hand sides). Here the three parameters S, epsilon and delta
// move together along their adjoint-state gradients: dJ/dS from the taped
// second solve, dJ/depsilon = dJ/dC11 2 C33 and dJ/ddelta = dJ/dC13 C33 (C33
// - C55) / (C13 + C55) (sf_batch_stiffness_gradient); each update is smoothed
// as the reference smooths dS, dE, dD (model_smoothing) and accepted when the
// misfit falls.
class Tomography_VTI : public Inversion
{
private:
    Eikonal_ANI* eikonal = nullptr;
    std::vector<float> E, D, dE, dD;
    void set_modeling_type() override;        // tomography_vti.cpp:3-22
    void export_estimated_models() override;  // tomography_vti.cpp:141-168

public:
    void optimization() override;
    void model_update() override;  // tomography_vti.cpp:121-139
};

#endif
