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

public:
    bool converged = false;
    std::string parameters;

    void set_parameters();     // inversion.cpp:3-22 (keys as written in run/parameters.txt)
    void import_obsData();     // inversion.cpp:24-50
    void forward_modeling();   // inversion.cpp:52-67: all shots in one taped launch
    void check_convergence();  // inversion.cpp:179-198
    void optimization();       // adjoint gradient + line search (replaces :200-345)
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

#endif
