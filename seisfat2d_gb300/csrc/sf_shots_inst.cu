// One instantiation of the forward kernel k_shots per object file: the build
// compiles this file once per variant with SF_TAPE, SF_REF, SF_INTERIOR,
// SF_COMP (true/false) and SF_KSHOTS_NAME set, in parallel, and the engine
// reaches each through its accessor (sf_kshots_kernel in sf_engine.cu).
#include "sf_forward.cuh"

#if !defined(SF_TAPE) || !defined(SF_REF) || !defined(SF_INTERIOR) || !defined(SF_COMP) || !defined(SF_KSHOTS_NAME)
#error "compile with -DSF_TAPE=.. -DSF_REF=.. -DSF_INTERIOR=.. -DSF_COMP=.. -DSF_KSHOTS_NAME=.."
#endif

namespace sf {

template __global__ void k_shots<SF_TAPE, SF_REF, SF_INTERIOR, SF_COMP>(FwdParams);

const void* SF_KSHOTS_NAME() { return (const void*)k_shots<SF_TAPE, SF_REF, SF_INTERIOR, SF_COMP>; }

}  // namespace sf
