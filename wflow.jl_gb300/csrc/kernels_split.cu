// kernels_split.cu -- FP32/FP64 split form (placeholder until the split kernels land).
#include "wf_kernels.h"

cudaError_t wf_split_vertical(const WfDevFields&, const WfLaunchCfg&) { return cudaErrorNotSupported; }
cudaError_t wf_split_ssf(const WfDevFields&, const WfDevGraph&, const WfSweep&, const WfLaunchCfg&) {
    return cudaErrorNotSupported;
}
cudaError_t wf_split_overland(const WfDevFields&, const WfDevGraph&, const WfSweep&, const WfLaunchCfg&) {
    return cudaErrorNotSupported;
}
cudaError_t wf_split_river(const WfDevFields&, const WfDevGraph&, const WfSweep&, const WfLaunchCfg&) {
    return cudaErrorNotSupported;
}
cudaError_t wf_split_balance(const WfDevFields&, const WfLaunchCfg&) { return cudaErrorNotSupported; }
