// refine_blocks.cu — the one-pass FP32 refine built for 6 resident
// 256-thread blocks per SM (40 registers: the form picked in build-major
// candidate order, where more resident warps hide the shared build
// geometry's load latency better than registers do); 4 lives in refine.cu.
#include "refine_eval.cuh"

namespace spj {

void launch_refine_blocks6(const RefineLaunch& a) {
  const uint32_t trips = a.m_dev ? 0 : kRefineChunkTrips;
  k_refine<true, 6><<<refine_grid(a.m, trips), 256, 0, a.s>>>(
      a.build, a.probe, a.cb, a.cp, a.m, a.probe_base, a.predicate, a.flags, a.st, a.m_dev,
      a.perm, nullptr, nullptr, nullptr, trips);
  SPJ_CUDA(cudaGetLastError());
}

}  // namespace spj
