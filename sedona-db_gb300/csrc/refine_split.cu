// refine_split.cu — the two-pass FP32 refine: a cheap pass over every pair
// (isolation exit, first vertex) that queues the pairs it leaves open, then
// the full evaluation of the queue (k_refine phases 1 and 2).
#include "refine_eval.cuh"

namespace spj {

void launch_refine_split(const RefineLaunch& a, int min_blocks, int group) {
  const int g = grid_for((int64_t)a.m, 256, kNumSMs * 16);
  SPJ_CUDA(cudaMemsetAsync(a.qn, 0, sizeof(uint32_t), a.s));
  if (group == 4 || group == 8 || group == 16) {
    // the cheap pass, then the queued pairs with `group` lanes each
    const int gg = grid_for((int64_t)a.m * group, 256, kNumSMs * 16);
    if (min_blocks == 6)
      k_refine<true, 6, 1><<<g, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m, a.probe_base,
                                               a.predicate, a.flags, a.st, a.m_dev, a.perm,
                                               a.queue, a.qn);
    else
      k_refine<true, 4, 1><<<g, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m, a.probe_base,
                                               a.predicate, a.flags, a.st, a.m_dev, a.perm,
                                               a.queue, a.qn);
#define SPJ_QGROUP(G)                                                                           \
  k_refine_group<G, 4, true><<<gg, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m, a.probe_base, \
                                                  a.predicate, a.flags, a.st, a.m_dev, a.queue,   \
                                                  a.qn)
    if (group == 4) {
      SPJ_QGROUP(4);
    } else if (group == 8) {
      SPJ_QGROUP(8);
    } else {
      SPJ_QGROUP(16);
    }
#undef SPJ_QGROUP
    SPJ_CUDA(cudaGetLastError());
    return;
  }
  if (min_blocks == 6) {
    k_refine<true, 6, 1><<<g, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m, a.probe_base,
                                             a.predicate, a.flags, a.st, a.m_dev, a.perm, a.queue,
                                             a.qn);
    k_refine<true, 6, 2><<<g, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m, a.probe_base,
                                             a.predicate, a.flags, a.st, a.m_dev, a.queue,
                                             a.queue, a.qn);
  } else {
    k_refine<true, 4, 1><<<g, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m, a.probe_base,
                                             a.predicate, a.flags, a.st, a.m_dev, a.perm, a.queue,
                                             a.qn);
    k_refine<true, 4, 2><<<g, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m, a.probe_base,
                                             a.predicate, a.flags, a.st, a.m_dev, a.queue,
                                             a.queue, a.qn);
  }
  SPJ_CUDA(cudaGetLastError());
}

}  // namespace spj
