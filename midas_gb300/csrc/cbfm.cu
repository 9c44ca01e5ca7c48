// cbfm.cu -- CBFM-E pipeline (placeholder until the batched implementation lands).
#include "common.cuh"
#include "kernels.cuh"

namespace midas {

int cbfm_run(midas_gpu_ctx *c, int, const int *, const int *, const int *, int, const double *, const double *, double,
             double, int, double, int, int, const double *, const double *, double2 *, int *, midas_gpu_info *)
{
    return c->err.set(MIDAS_ERR_UNSUPPORTED, "cbfm_solve: not built yet");
}

int aca_run(midas_gpu_ctx *c, int, int, int, int, double, int, double2 *, double2 *, int *)
{
    return c->err.set(MIDAS_ERR_UNSUPPORTED, "aca: not built yet");
}

}  // namespace midas
