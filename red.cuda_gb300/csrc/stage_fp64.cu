// stage_fp64.cu -- k_stage instantiated for mode FP64: every pair in FP64 with FMA.
// One translation unit per mode keeps the parallel build short; each unit
// holds its own copy of the Butcher tableau in constant memory.
#include "stage.cuh"

namespace redgb {

void set_tableau_fp64(const Tableau& tb, cudaStream_t s)
{
    cudaMemcpyToSymbolAsync(c_tb, &tb, sizeof(Tableau), 0, cudaMemcpyHostToDevice, s);
}

void launch_stage_fp64(const StageParams& P, int n, int variant, cudaStream_t s)
{
    launch_stage_variant<MODE_FP64, false>(P, n, variant, s);
}

}  // namespace redgb
