// refine_blocks.cu — the one-pass FP32 refine built for 2, 3, 5 or 6
// resident 256-thread blocks per SM (the register budget trades against the
// number of warps that hide load latency); 4 lives in refine.cu.
#include "refine_eval.cuh"

namespace spj {

void launch_refine_blocks(const RefineLaunch& a, int min_blocks) {
  const int g = grid_for((int64_t)a.m, 256, kNumSMs * 16);
#define SPJ_BLOCKS_LAUNCH(MB)                                                                \
  k_refine<true, MB><<<g, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m, a.probe_base, \
                                         a.predicate, a.flags, a.st, a.m_dev, a.perm)
  if (min_blocks == 6) SPJ_BLOCKS_LAUNCH(6);
  else if (min_blocks == 5) SPJ_BLOCKS_LAUNCH(5);
  else if (min_blocks == 3) SPJ_BLOCKS_LAUNCH(3);
  else SPJ_BLOCKS_LAUNCH(2);
#undef SPJ_BLOCKS_LAUNCH
  SPJ_CUDA(cudaGetLastError());
}

}  // namespace spj
