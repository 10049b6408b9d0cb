// stage_exact.cu -- k_stage instantiated for mode FP64_EXACT: red's operation order, bit-identical to its CPU code.
// One translation unit per mode keeps the parallel build short; each unit
// holds its own copy of the Butcher tableau in constant memory.
#include "stage.cuh"

namespace redgb {

void set_tableau_exact(const Tableau& tb, cudaStream_t s)
{
    cudaMemcpyToSymbolAsync(c_tb, &tb, sizeof(Tableau), 0, cudaMemcpyHostToDevice, s);
}

void launch_stage_exact(const StageParams& P, int n, int variant, cudaStream_t s)
{
    launch_stage_variant<MODE_FP64_EXACT, true>(P, n, variant, s);
}

}  // namespace redgb
