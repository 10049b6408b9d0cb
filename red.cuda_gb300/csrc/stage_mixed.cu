// stage_mixed.cu -- k_stage instantiated for mode MIXED: double-single FP32 body-body pairs, FP64 star term.
// One translation unit per mode keeps the parallel build short; each unit
// holds its own copy of the Butcher tableau in constant memory.
#include "stage.cuh"

namespace redgb {

void set_tableau_mixed(const Tableau& tb, cudaStream_t s)
{
    cudaMemcpyToSymbolAsync(c_tb, &tb, sizeof(Tableau), 0, cudaMemcpyHostToDevice, s);
}

void launch_stage_mixed(const StageParams& P, int n, int variant, cudaStream_t s)
{
    launch_stage_variant<MODE_MIXED, false>(P, n, variant, s);
}

int active_clusters_mixed() { return stage_active_clusters<MODE_MIXED, false>(); }

}  // namespace redgb
