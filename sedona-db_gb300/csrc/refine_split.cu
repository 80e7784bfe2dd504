// refine_split.cu — the two-pass FP32 refine: a cheap pass over every pair
// (isolation exit, first vertex) that queues the pairs it leaves open, then
// the full evaluation of the queue (k_refine phases 1 and 2).  Ordered: the
// cheap pass queues slots of the candidate permutation, which are sorted back
// into its order, so the full pass takes the open pairs in build-major order.
#include "prims.cuh"
#include "refine_eval.cuh"

namespace spj {

namespace {
template <int MB>
void split_passes(const RefineLaunch& a, int g, const uint32_t* slot_perm, bool sort_queue) {
  k_refine<true, MB, 1><<<g, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m, a.probe_base,
                                            a.predicate, a.flags, a.st, a.m_dev, a.perm, a.queue,
                                            a.qn, slot_perm);
  SPJ_CUDA(cudaGetLastError());
  if (sort_queue) {
    uint32_t nq = 0;
    SPJ_CUDA(cudaMemcpyAsync(&nq, a.qn, sizeof nq, cudaMemcpyDeviceToHost, a.s));
    SPJ_CUDA(cudaStreamSynchronize(a.s));
    if (nq > 1) {
      int bits = 1;
      while (bits < 32 && (a.m - 1) >> bits) bits++;
      DevBuf vals((size_t)nq * 4, a.s), ak((size_t)nq * 4, a.s), av((size_t)nq * 4, a.s), tmp;
      radix_sort_pairs(a.queue, vals.as<uint32_t>(), ak.as<uint32_t>(), av.as<uint32_t>(), nq,
                       bits, tmp, a.s);
    }
  }
  k_refine<true, MB, 2><<<g, 256, 0, a.s>>>(a.build, a.probe, a.cb, a.cp, a.m, a.probe_base,
                                            a.predicate, a.flags, a.st, a.m_dev, a.queue, a.queue,
                                            a.qn, slot_perm);
  SPJ_CUDA(cudaGetLastError());
}
}  // namespace

void launch_refine_split(const RefineLaunch& a, int min_blocks, bool ordered) {
  const int g = grid_for((int64_t)a.m, 256, kNumSMs * 16);
  SPJ_CUDA(cudaMemsetAsync(a.qn, 0, sizeof(uint32_t), a.s));
  // (ordering needs a permutation whose slots are all candidates, and a host
  // read of the queue length: not inside a graph capture, so not with m_dev)
  const bool sort_queue = ordered && a.perm != nullptr && a.m_dev == nullptr;
  const uint32_t* slot_perm = sort_queue ? a.perm : nullptr;
  if (min_blocks == 6) split_passes<6>(a, g, slot_perm, sort_queue);
  else split_passes<4>(a, g, slot_perm, sort_queue);
}

}  // namespace spj
