// refine_split.cu — the two-pass FP32 refine: a cheap pass over every pair
// (isolation exit, first vertex) that queues the pairs it leaves open, then
// the full evaluation of the queue (k_refine phases 1 and 2).
#include "refine_eval.cuh"

namespace spj {

void launch_refine_split(const RefineLaunch& a, int min_blocks) {
  const int g = grid_for((int64_t)a.m, 256, kNumSMs * 16);
  SPJ_CUDA(cudaMemsetAsync(a.qn, 0, sizeof(uint32_t), a.s));
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
