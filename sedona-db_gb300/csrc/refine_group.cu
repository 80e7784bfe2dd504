// refine_group.cu — the group-cooperative FP32 refine: kG lanes per
// candidate pair split the ring loops (k_refine_group).
#include "refine_eval.cuh"

namespace spj {

void launch_refine_group(const RefineLaunch& a, int group, int min_blocks) {
  const int gg = grid_for((int64_t)a.m * group, 256, kNumSMs * 16);
#define SPJ_GROUP_LAUNCH(G, MB)                                                              \
  k_refine_group<G, MB><<<gg, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m, a.probe_base, \
                                             a.predicate, a.flags, a.st, a.m_dev)
  const bool wide = min_blocks <= 2;  // 128 registers, two blocks per SM
  if (group == 4) {
    if (wide) SPJ_GROUP_LAUNCH(4, 2);
    else SPJ_GROUP_LAUNCH(4, 4);
  } else if (group == 8) {
    if (wide) SPJ_GROUP_LAUNCH(8, 2);
    else SPJ_GROUP_LAUNCH(8, 4);
  } else {
    if (wide) SPJ_GROUP_LAUNCH(16, 2);
    else SPJ_GROUP_LAUNCH(16, 4);
  }
#undef SPJ_GROUP_LAUNCH
  SPJ_CUDA(cudaGetLastError());
}

}  // namespace spj
