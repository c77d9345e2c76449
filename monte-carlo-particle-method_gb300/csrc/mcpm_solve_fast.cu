// mcpm_solve_fast.cu -- the FP32 sessions' per-cell solve (k_solve<false>).
//
// The same kernel source as the exact FP64 path (mcpm_solve.cuh), compiled
// with --fmad=true: its multiply-adds contract into DFMA instructions.  The
// kernel runs on GB300's FP64 pipe (one DFMA, DADD or DMUL per pipe slot),
// so every contracted pair is a pipe slot saved.  The FP32 sessions' results
// are rounded to float for the particle pass, and the contraction only makes
// their FP64 intermediates more accurate; the FP64 sessions keep the
// reference's separate roundings (mcpm_kernels.cu, --fmad=false).
// 4 blocks of 128 threads per SM (128 registers a thread, the rest in
// local memory): measured 3 % faster than 2 blocks at 255 registers
#define MCPM_SOLVE_MINB 4
#include "mcpm_solve.cuh"

namespace mcpm {

int launch_solve_fast(Session& s, int with_alpha, int fp_model) {
  const int bt = solve_block(s), nb = (s.C + bt - 1) / bt;
  k_solve<false><<<nb, bt, 0, s.stream>>>(s.k, s.cell, s.pcell, with_alpha, fp_model, s.status);
  return 1;
}

}  // namespace mcpm
