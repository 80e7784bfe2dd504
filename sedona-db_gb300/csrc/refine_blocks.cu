// refine_blocks.cu — the one-pass FP32 refine built for 6 resident
// 256-thread blocks per SM (40 registers: the form picked in build-major
// candidate order, where more resident warps hide the shared build
// geometry's load latency better than registers do); 4 lives in refine.cu.
#include "refine_eval.cuh"

namespace spj {

void launch_refine_blocks6(const RefineLaunch& a) {
  if (a.chunk_trips && a.m_dev == nullptr) {
    // one block per chunk_trips x 256 consecutive slots
    const uint64_t per = 256ull * a.chunk_trips;
    const uint64_t g = (a.m + per - 1) / per;
    k_refine<true, 6><<<(unsigned)g, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m,
                                                     a.probe_base, a.predicate, a.flags, a.st,
                                                     a.m_dev, a.perm, nullptr, nullptr, nullptr,
                                                     a.chunk_trips);
  } else {
    const int g = grid_for((int64_t)a.m, 256, kNumSMs * 16);
    k_refine<true, 6><<<g, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m, a.probe_base,
                                          a.predicate, a.flags, a.st, a.m_dev, a.perm);
  }
  SPJ_CUDA(cudaGetLastError());
}

}  // namespace spj
