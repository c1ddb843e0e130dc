// wg_kernels.h -- launchers of the kernels in wg_kernels.cu (host side).
#pragma once
#include <cuda_runtime.h>

#include "wg_device.h"

namespace wg {
cudaError_t launch_vertical(const DevCells &c, const DevState &s, const DevVert &v, const DevForcing &f, int doy,
                            int fday, cudaStream_t st);
int pipeline_max_blocks(bool fused);
cudaError_t launch_pipeline(bool fused, const DevCells &c, const DevState &s, const DevVert &v, const DevForcing &f,
                            const DevBalance &b, const DevSync &sync, double *outq, double *qst, int doy0, int fday0,
                            int oday0, int ndays, int blocks, cudaStream_t st);
cudaError_t launch_volume(const DevCells &c, const DevState &s, double *vol, cudaStream_t st);
cudaError_t launch_balance_sum(const DevCells &c, const DevState &s, const DevBalance &b, const double *vol0,
                               double *partial, int *nblocks, cudaStream_t st);
}  // namespace wg
