// kernels.h -- host-side launchers of the sm_103a kernels (eval_kernels.cu,
// switch_kernels.cu).  All launchers are asynchronous on the given stream.
#ifndef PSI_KERNELS_H
#define PSI_KERNELS_H

#include <cstdint>
#include <cuda_runtime.h>

namespace psi {

// ---- strategy set-up (gpu_parity.cu:38-56, cpu_parity.cpp:276-286, 300-307)
void launch_init_strat(cudaStream_t s, int32_t n, const int8_t *owner, const int32_t *off,
                       const int32_t *tgt, int32_t *strat, int32_t *st);
void launch_reset_odd(cudaStream_t s, int32_t n, const int8_t *owner, const int32_t *off,
                      const int32_t *tgt, int32_t *strat);

// ---- evaluation: Euler tour, Helman-JaJa sublists, Wyllie on the reduced list
void launch_tour_init(cudaStream_t s, int32_t n, int32_t *succ, int2 *vloc);
void launch_tour_link(cudaStream_t s, int32_t n, const int32_t *strat, const uint8_t *solved,
                      int32_t *succ);
void launch_pick_heads(cudaStream_t s, int64_t L, int32_t nsub, int32_t stride, int32_t *succ,
                       int32_t *hsucc);
void launch_walk_sublists(cudaStream_t s, int32_t nsub, int32_t n, int64_t L, const int32_t *succ,
                          const int32_t *hsucc, int2 *vloc, int2 *red, uint32_t *err);
void launch_wyllie_round(cudaStream_t s, int32_t nsub, const int2 *in, int2 *out);
void launch_broadcast_depth(cudaStream_t s, int32_t n, const int2 *vloc, const int2 *red,
                            const int32_t *strat, const int32_t *pri, const uint8_t *solved,
                            int32_t *st, int2 *pp, int32_t *ulist, int32_t *ucount);
// ---- cycle parity of the vertices the sink does not reach (pointer jumping)
void launch_jump_init(cudaStream_t s, int32_t nu, const int32_t *ulist, const int32_t *strat,
                      const int32_t *pri, int2 *jmp, uint32_t *err);
void launch_jump_round(cudaStream_t s, int32_t nu, const int32_t *ulist, const uint8_t *solved,
                       const int2 *in, int2 *out);
void launch_jump_finish(cudaStream_t s, int32_t nu, const int32_t *ulist, const uint8_t *solved,
                        const int2 *jmp, int32_t *st);
void launch_mark_solved(cudaStream_t s, int32_t n, int32_t player, const int32_t *st,
                        uint8_t *solved);

// ---- all-switches (gpu_parity.cu:191-317, cpu_parity.cpp:154-263)
void launch_switch(cudaStream_t s, int32_t n, int32_t player, const int8_t *owner,
                   const int32_t *off, const int32_t *tgt, int32_t *strat, const int32_t *st,
                   const int2 *pp, unsigned long long *count, uint32_t *err);
// ---- dense valuation rows for export (the reference's ArrayVal layout)
void launch_materialize(cudaStream_t s, int32_t v0, int32_t count, int32_t d, const int32_t *st,
                        const int2 *pp, int32_t *rows, uint32_t *err);

}  // namespace psi

#endif
