#include "modeling.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <iostream>
#include <stdexcept>
#include <vector>

#include "admin.hpp"

static void cuda_check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

// modeling.cu:3-36
void Modeling::set_parameters()
{
    nx = std::stoi(catch_parameter("x_samples", parameters));
    nz = std::stoi(catch_parameter("z_samples", parameters));
    dx = std::stof(catch_parameter("x_spacing", parameters));
    dz = std::stof(catch_parameter("z_spacing", parameters));
    data_folder = catch_parameter("modeling_output_folder", parameters);
    Cijkl_folder = catch_parameter("Cijkl_folder", parameters);

    nPoints = nx * nz;
    nb = 3;
    nxx = nx + 2 * nb;
    nzz = nz + 2 * nb;
    matsize = nxx * nzz;
    nBlocks = (matsize + 255) / 256;

    set_geometry();
    set_properties();
    create_engine();
    set_conditions();
    set_eikonal();
}

void Modeling::create_engine()
{
    if (ctx) return;
    sf_check(sf_ctx_create(&ctx, nx, nz, dx, dz, 0), nullptr, "sf_ctx_create");
    // eikonal_arithmetic = reference (default) | ieee | compensated (sf_set_arithmetic)
    std::string arith = catch_parameter("eikonal_arithmetic", parameters);
    if (arith == "ieee") sf_check(sf_set_arithmetic(ctx, SF_ARITH_IEEE), ctx, "sf_set_arithmetic");
    if (arith == "compensated") sf_check(sf_set_arithmetic(ctx, SF_ARITH_COMPENSATED), ctx, "sf_set_arithmetic");
}

void Modeling::set_geometry()
{
    delete geometry;
    geometry = new Geometry();
    geometry->parameters = parameters;
    geometry->set_parameters();
    delete[] seismogram;
    seismogram = new float[geometry->nrec]();
}

// modeling.cu:47-60
void Modeling::set_properties()
{
    std::vector<float> s(nPoints);
    import_binary_float(catch_parameter("slowness_file", parameters), s.data(), nPoints);
    delete[] S;
    S = new float[matsize]();
    expand_boundary(s.data(), S);
}

// modeling.cu:62-102: sizes and device buffers; the sign tables of the
// reference's launch loop live inside the engine's sweep kernel.
void Modeling::set_eikonal()
{
    dz2i = 1.0f / (dz * dz);
    dx2i = 1.0f / (dx * dx);
    total_levels = (nxx - 1) + (nzz - 1);
    delete[] T;
    T = new float[matsize]();
    if (!d_T) cuda_check(cudaMalloc((void**)&d_T, matsize * sizeof(float)), "cudaMalloc");
    if (!d_S) cuda_check(cudaMalloc((void**)&d_S, matsize * sizeof(float)), "cudaMalloc");
    copy_slowness_to_device();
}

void Modeling::set_shot_point()
{
    sx = geometry->xsrc[srcId];
    sz = geometry->zsrc[srcId];
}

// modeling.cu:110-121: the source node; the 3x3 start values are set inside
// the engine's solve.
void Modeling::initialization()
{
    sIdx = (int)((sx + 0.5f * dx) / dx) + nb;
    sIdz = (int)((sz + 0.5f * dz) / dz) + nb;
}

// modeling.cu:123-159: the whole 4-sweep solve (both solves and the qP pass
// for the anisotropic model) in one engine call on the engine's stream.
void Modeling::eikonal_solver()
{
    sf_check(sf_time_propagation(ctx, ani, sx, sz, d_T, SF_MEM_DEVICE, nullptr), ctx, "sf_time_propagation");
    sf_check(sf_synchronize(ctx, nullptr), ctx, "sf_synchronize");
}

// modeling.cu:161-194: picks on the device, host T refreshed for the callers
// that read it (Inversion, Migration).
void Modeling::compute_seismogram()
{
    sf_check(sf_compute_seismogram(ctx, d_T, geometry->xrec, geometry->zrec, geometry->nrec, seismogram,
                                   SF_MEM_HOST, nullptr),
             ctx, "sf_compute_seismogram");
    cuda_check(cudaMemcpy(T, d_T, matsize * sizeof(float), cudaMemcpyDeviceToHost), "cudaMemcpy");
}

// modeling.cu:196-202
void Modeling::export_seismogram()
{
    compute_seismogram();
    std::string data_file = data_folder + modeling_type + "_nStations" + std::to_string(geometry->nrec) +
                            "_shot_" + std::to_string(srcId + 1) + ".bin";
    export_binary_float(data_file, seismogram, geometry->nrec);
}

// modeling.cu:204-232
void Modeling::expand_boundary(float* input, float* output)
{
    for (int index = 0; index < nPoints; index++) {
        int i = index % nz, j = index / nz;
        output[(i + nb) + (j + nb) * nzz] = input[i + j * nz];
    }
    for (int i = 0; i < nb; i++)
        for (int j = nb; j < nxx - nb; j++) {
            output[i + j * nzz] = output[nb + j * nzz];
            output[(nzz - i - 1) + j * nzz] = output[(nzz - nb - 1) + j * nzz];
        }
    for (int i = 0; i < nzz; i++)
        for (int j = 0; j < nb; j++) {
            output[i + j * nzz] = output[i + nb * nzz];
            output[i + (nxx - j - 1) * nzz] = output[i + (nxx - nb - 1) * nzz];
        }
}

// modeling.cu:234-244
void Modeling::reduce_boundary(float* input, float* output)
{
    for (int index = 0; index < nPoints; index++) {
        int i = index % nz, j = index / nz;
        output[i + j * nz] = input[(i + nb) + (j + nb) * nzz];
    }
}

// modeling.cu:246-262 (without clearing the terminal)
void Modeling::show_information()
{
    std::cout << "SeisFAT2D (GB300 engine) | model (z = " << (nz - 1) * dz << ", x = " << (nx - 1) * dx
              << ") m | shot " << srcId + 1 << " of " << geometry->nsrc << " at (z = " << geometry->zsrc[srcId]
              << ", x = " << geometry->xsrc[srcId] << ") m | " << modeling_name << "\n";
}

void Modeling::compression(float* input, uintc* output, int N, float& max_value, float& min_value)
{
    max_value = -1e20f;
    min_value = 1e20f;
    for (int index = 0; index < N; index++) {
        min_value = std::fmin(input[index], min_value);
        max_value = std::fmax(input[index], max_value);
    }
    for (int index = 0; index < N; index++) {
        if (max_value == min_value) {
            output[index] = 1;
            continue;
        }
        output[index] = (uintc)(1.0f + (float)(65535 - 1) * (input[index] - min_value) / (max_value - min_value));
    }
}

// modeling.cu:281-284
void Modeling::copy_slowness_to_device()
{
    sf_check(sf_set_slowness(ctx, S, SF_LAYOUT_PADDED, SF_MEM_HOST), ctx, "sf_set_slowness");
    cuda_check(cudaMemcpy(d_S, S, matsize * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy");
}

Modeling::~Modeling()
{
    if (ctx) sf_ctx_destroy(ctx);
    if (d_T) cudaFree(d_T);
    if (d_S) cudaFree(d_S);
    delete[] S;
    delete[] T;
    delete[] seismogram;
    delete geometry;
}

// ---------------------------------------------------------------- Eikonal_ISO

void Eikonal_ISO::set_conditions()
{
    modeling_type = "eikonal_iso";
    modeling_name = "Modeling type: Eikonal isotropic solver";
    ani = 0;
}

void Eikonal_ISO::time_propagation()
{
    initialization();
    eikonal_solver();
}

// ---------------------------------------------------------------- Eikonal_ANI

// eikonal_ani.cu:3-16: one Cij field, padded; quantised by the engine
void Eikonal_ANI::set_stiffness_element(std::string element, float* padded)
{
    std::vector<float> aux(nPoints);
    import_binary_float(Cijkl_folder + element + ".bin", aux.data(), nPoints);
    expand_boundary(aux.data(), padded);
}

void Eikonal_ANI::set_conditions()
{
    modeling_type = "eikonal_ani";
    modeling_name = "Modeling type: Anisotropic eikonal solver";
    ani = 1;
    const char* names[6] = {"C11", "C13", "C15", "C33", "C35", "C55"};
    for (int q = 0; q < 6; q++) {
        cij[q].assign(matsize, 0.0f);
        set_stiffness_element(names[q], cij[q].data());
    }
    upload_stiffness();
}

// modeling.cu:264-279 on each padded field, then the codes to the engine
void Eikonal_ANI::upload_stiffness()
{
    std::vector<std::vector<uintc>> codes(6, std::vector<uintc>(matsize));
    float mm[12];
    const uint16_t* cp[6];
    for (int q = 0; q < 6; q++) {
        compression(cij[q].data(), codes[q].data(), matsize, mm[2 * q + 1], mm[2 * q]);
        cp[q] = codes[q].data();
    }
    sf_check(sf_set_stiffness_codes(ctx, cp, mm, SF_MEM_HOST), ctx, "sf_set_stiffness_codes");
}

// epsilon = (C11 - C33) / (2 C33), delta = ((C13 + C55)^2 - (C33 - C55)^2) /
// (2 C33 (C33 - C55)): the inverse of the VTI relations of
// src/functions.py:72-109
void Eikonal_ANI::get_stiffness_VTI(float* E, float* D) const
{
    for (int index = 0; index < nPoints; index++) {
        const int i = index % nz + nb, j = index / nz + nb;
        const size_t k = (size_t)i + (size_t)j * nzz;
        const double c11 = cij[0][k], c13 = cij[1][k], c33 = cij[3][k], c55 = cij[5][k];
        E[index] = (float)((c11 - c33) / (2.0 * c33));
        D[index] = (float)(((c13 + c55) * (c13 + c55) - (c33 - c55) * (c33 - c55)) / (2.0 * c33 * (c33 - c55)));
    }
}

// C11 = C33 (1 + 2 epsilon), C13 = sqrt((C33 - C55)(2 delta C33 + C33 - C55))
// - C55 on the model cells (delta held where the root stays real), padded by
// edge replication, quantised and uploaded
void Eikonal_ANI::set_stiffness_VTI(const float* E, const float* D)
{
    std::vector<float> m11(nPoints), m13(nPoints);
    for (int index = 0; index < nPoints; index++) {
        const int i = index % nz + nb, j = index / nz + nb;
        const size_t k = (size_t)i + (size_t)j * nzz;
        const double c33 = cij[3][k], c55 = cij[5][k];
        const double arg = (c33 - c55) * (2.0 * (double)D[index] * c33 + c33 - c55);
        m11[index] = (float)(c33 * (1.0 + 2.0 * (double)E[index]));
        m13[index] = (float)(std::sqrt(std::max(arg, 0.0)) - c55);
    }
    expand_boundary(m11.data(), cij[0].data());
    expand_boundary(m13.data(), cij[1].data());
    upload_stiffness();
}

void Eikonal_ANI::time_propagation()
{
    initialization();
    eikonal_solver();
}
