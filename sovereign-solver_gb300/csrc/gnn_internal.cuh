// gnn_internal.cuh — what other translation units of the library may use of a
// warm-start network object (sps_gnn, defined in gnn.cu): its device input and
// output buffers and a forward pass on inputs already in place.  Used by the
// batched solver to predict warm starts without leaving the device.
#pragma once

#include <cuda_runtime.h>

#include "../../include/sps_gnn.h"

namespace sps {
namespace gnn {

struct DeviceIO {
    int n, m, max_batch, lp_features, device;
    cudaStream_t stream;
    float *c_in, *b_in;                 // lp_features inputs (max_batch x n, max_batch x m)
    const float *x0, *y0, *log_omega;   // outputs of the last forward
};

int device_io(sps_gnn* g, DeviceIO* io);
// Forward pass of `batch` instances whose inputs are already in c_in / b_in
// (queued on io.stream; no synchronisation).
int forward_in_place(sps_gnn* g, int batch);
// After the network's stream is synchronised: 0, or the internal error of a
// tensor-core node update that gave up waiting (that forward's outputs are invalid).
int check_device_error(sps_gnn* g);

}  // namespace gnn
}  // namespace sps
