// proposer.cuh -- layout of the learned step proposer (proposer.cu).
#pragma once
#include <cuda_bf16.h>

#include "redgb_dev.cuh"

namespace redgb {

constexpr int kFeat = 12;      // features per system
constexpr int kLogRec = kFeat + 2;   // floats per logged record: features, log|dt|, log(err / tol)
constexpr int kHid = 64;       // hidden width of both layers
// parameters, flat: W1[kHid][kFeat], b1[kHid], W2[kHid][kHid], b2[kHid], w3[kHid], b3
constexpr int oW1 = 0;
constexpr int oB1 = oW1 + kHid * kFeat;
constexpr int oW2 = oB1 + kHid;
constexpr int oB2 = oW2 + kHid * kHid;
constexpr int oW3 = oB2 + kHid;
constexpr int oB3 = oW3 + kHid;
constexpr int kNParam = oB3 + 1;   // 5057
constexpr int kNPart = 10;     // partial sums per feature segment
constexpr int kTrainRows = 16; // rows per CTA of the training kernel

struct MlpNorm {
    float x_mean[kFeat], x_std[kFeat];
    float y_mean, y_std;
};

struct FeatParams {
    const Segment* segs;
    const SysInfo* sinfo;
    const DevSys* sys;
    const float4* pos;     // FP32 hi words of the accepted state's positions
    const double* y_v;
    const double* acc;     // stage-0 accelerations of the accepted try
    const double* mass;
    const int* id;
    float* part;           // kNPart per segment
};

struct ProposeParams {
    int n_sys;
    DevSys* sys;
    const int* seg0;       // first feature segment of each system
    const int* nseg;
    const float* part;
    double tolerance;
    int propose;           // 1: the MLP sets the next try's step
    const __nv_bfloat16* w;
    MlpNorm norm;
    double safety, ratio_lo, ratio_hi, output_interval;
    int log;               // 1: append (previous features, log|dt| accepted) records
    float* feat_prev;      // kFeat per system
    int* has_prev;
    float* log_buf;        // (kFeat + 1) floats per record
    unsigned int* log_n;
    unsigned int log_cap;
};

void launch_features(const FeatParams& F, int n_segs, cudaStream_t s);
void launch_propose(const ProposeParams& P, cudaStream_t s);

}  // namespace redgb
