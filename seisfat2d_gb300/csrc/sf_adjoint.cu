// Adjoint-state gradient of the pick misfit (entry points; kernels follow).
#include <cuda_runtime.h>

#include "sf_engine.h"

void sf_adjoint_release(sf_ctx* c)
{
    void* bufs[] = {c->d_lam, c->d_vrec, c->d_gshot, c->d_pg, c->d_misfit, c->d_colshots, c->d_colptr};
    for (void* b : bufs)
        if (b) cudaFree(b);
}

extern "C" int sf_batch_adjoint(sf_ctx* c, const float*, int, float*, int, void*)
{
    return sf_fail(c, SF_ERR_STATE, "adjoint not available");
}

extern "C" int sf_batch_misfit_gradient(sf_ctx* c, const float*, int, double*, float*, int, void*)
{
    return sf_fail(c, SF_ERR_STATE, "adjoint not available");
}
