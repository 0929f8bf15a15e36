// Drop-in for the reference's Modeling class hierarchy
// (src/modeling/modeling.cuh:17-79, eikonal_iso.cuh, eikonal_ani.cuh): the same
// public members and methods with the same meaning, backed by the GB300
// engine's C ABI (include/seisfat2d.h). After time_propagation() d_T holds the
// padded traveltimes (nzz x nxx, z fastest) on the device; after
// compute_seismogram() the host T holds them too and seismogram[] the picks.
#ifndef SF_HOST_MODELING_HPP
#define SF_HOST_MODELING_HPP

#include <cstdint>
#include <string>
#include <vector>

#include "geometry.hpp"
#include "seisfat2d.h"

typedef unsigned short int uintc;  // modeling.cuh:15

class Modeling
{
private:
    void set_properties();
    void create_engine();

protected:
    int total_levels = 0;
    float dx2i = 0.0f, dz2i = 0.0f;

    sf_ctx* ctx = nullptr;  // the engine context that replaces d_sgnv/d_sgnt and the launch loop
    int ani = 0;            // 1 for the two-pass anisotropic solve

    // modeling.cu:264-279 with a deterministic min/max
    void compression(float* input, uintc* output, int N, float& max_value, float& min_value);

public:
    float dx = 0.0f, dz = 0.0f;
    int nxx = 0, nzz = 0, matsize = 0;
    int nx = 0, nz = 0, nb = 3, nPoints = 0;
    int srcId = 0, recId = 0, sIdx = 0, sIdz = 0;
    int nBlocks = 0;

    float sx = 0.0f, sz = 0.0f;

    float* S = nullptr;
    float* T = nullptr;

    float* d_T = nullptr;
    float* d_S = nullptr;

    float* seismogram = nullptr;

    Geometry* geometry = nullptr;

    std::string parameters;
    std::string data_folder;
    std::string modeling_type;
    std::string modeling_name;
    std::string Cijkl_folder;

    void set_eikonal();
    void set_geometry();

    void set_parameters();
    void initialization();
    void eikonal_solver();
    void set_shot_point();
    void show_information();
    void compute_seismogram();

    void copy_slowness_to_device();

    void expand_boundary(float* input, float* output);
    void reduce_boundary(float* input, float* output);

    virtual void set_conditions() = 0;
    virtual void time_propagation() = 0;

    void export_seismogram();

    sf_ctx* engine() const { return ctx; }
    int anisotropic() const { return ani; }
    virtual ~Modeling();
};

class Eikonal_ISO : public Modeling
{
public:
    void set_conditions() override;    // eikonal_iso.cu:3-7
    void time_propagation() override;  // eikonal_iso.cu:9-12
};

class Eikonal_ANI : public Modeling
{
private:
    void set_stiffness_element(std::string element, float* padded);
    void upload_stiffness();

    // padded C11, C13, C15, C33, C35, C55 (nzz x nxx), as last uploaded
    std::vector<float> cij[6];

public:
    void set_conditions() override;    // eikonal_ani.cu:18-31
    void time_propagation() override;  // eikonal_ani.cu:33-45

    // Thomsen epsilon and delta (nz x nx) of the loaded stiffness, and the
    // stiffness rebuilt from them with C33 and C55 kept: the two calls
    // Tomography_VTI makes (tomography_vti.cpp:22, :128), which the
    // reference never defines. VTI only (C15 and C35 are kept as loaded).
    void get_stiffness_VTI(float* E, float* D) const;
    void set_stiffness_VTI(const float* E, const float* D);
    const std::vector<float>& stiffness(int q) const { return cij[q]; }
};

#endif
