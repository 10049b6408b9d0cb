// stage_fp32.cu -- k_stage instantiated for mode FP32: plain FP32 coordinates, FP64 star term.
// One translation unit per mode keeps the parallel build short; each unit
// holds its own copy of the Butcher tableau in constant memory.
#include "stage.cuh"

namespace redgb {

void set_tableau_fp32(const Tableau& tb, cudaStream_t s)
{
    cudaMemcpyToSymbolAsync(c_tb, &tb, sizeof(Tableau), 0, cudaMemcpyHostToDevice, s);
}

void launch_stage_fp32(const StageParams& P, int n, int variant, cudaStream_t s)
{
    launch_stage_variant<MODE_FP32, false>(P, n, variant, s);
}

int active_clusters_fp32() { return stage_active_clusters<MODE_FP32, false>(); }

}  // namespace redgb
