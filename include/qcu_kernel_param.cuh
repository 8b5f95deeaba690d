/*
 * qcu_kernel_param.cuh -- the stream set of the reference's C++ interface
 * (include/qcu_kernel_param.cuh:9-38 of the reference): one compute stream
 * and eight boundary streams (4 dimensions x 2 directions), in that order,
 * so an object built against either header passes by reference.  The
 * dslash entry points run on `stream` and return when it has finished.
 *
 * Differences kept out of the shared layout: a stream that cannot be
 * created is left as the legacy default stream (0) instead of terminating
 * the process, and a copy shares the streams without destroying them (the
 * reference's copies destroy the same streams twice).
 */
#pragma once

#include <cuda_runtime.h>

namespace qcu {

struct ExecutionStreams {
  cudaStream_t stream;
  cudaStream_t boundaryStreams[4 * 2];  // 4 dims, 2 dirs

  ExecutionStreams() : owner_(true) {
    if (cudaStreamCreate(&stream) != cudaSuccess) stream = 0;
    for (int i = 0; i < 4 * 2; i++)
      if (cudaStreamCreate(&boundaryStreams[i]) != cudaSuccess) boundaryStreams[i] = 0;
  }
  ExecutionStreams(const ExecutionStreams &o) : owner_(false) { share(o); }
  void operator=(const ExecutionStreams &o) {
    release();
    share(o);
    owner_ = false;
  }
  ~ExecutionStreams() { release(); }

 private:
  bool owner_;  // after the reference's members: code built against either header reads the same offsets
  void share(const ExecutionStreams &o) {
    stream = o.stream;
    for (int i = 0; i < 4 * 2; i++) boundaryStreams[i] = o.boundaryStreams[i];
  }
  void release() {
    if (!owner_) return;
    if (stream) cudaStreamDestroy(stream);
    for (int i = 0; i < 4 * 2; i++)
      if (boundaryStreams[i]) cudaStreamDestroy(boundaryStreams[i]);
    owner_ = false;
  }
};

}  // namespace qcu
