// mcpm_surrogate.h -- parameter layout and launchers of the learned Vlasov
// force (mcpm_surrogate.cu, mcpm_surrogate_tc.cu).
#pragma once
#include <cstdint>
#include <string>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace mcpm {

// fp32 parameter array: conv weights [co][tap][ci] (tap = 3 (dy + 1) + dx + 1)
// and biases; layer 1 reads 16 input channels, layer 4 writes 16 outputs
// (only the first 4 are used; the other rows stay zero under training
// because their gradients are zero).
enum : int {
  SP_W = 64,
  SP_CIN = 16,
  SP_COUT = 16,
  SP_OFF_W1 = 0,
  SP_OFF_B1 = SP_OFF_W1 + SP_W * 9 * SP_CIN,
  SP_OFF_W2 = SP_OFF_B1 + SP_W,
  SP_OFF_B2 = SP_OFF_W2 + SP_W * 9 * SP_W,
  SP_OFF_W3 = SP_OFF_B2 + SP_W,
  SP_OFF_B3 = SP_OFF_W3 + SP_W * 9 * SP_W,
  SP_OFF_W4 = SP_OFF_B3 + SP_W,
  SP_OFF_B4 = SP_OFF_W4 + SP_COUT * 9 * SP_W,
  SP_NPARAM = SP_OFF_B4 + SP_COUT,
  // transposed, tap-flipped bf16 weights of the data-gradient convolutions
  SF_OFF_F4 = 0,                          // [64][9][16]
  SF_OFF_F3 = SF_OFF_F4 + SP_W * 9 * SP_COUT,  // [64][9][64]
  SF_OFF_F2 = SF_OFF_F3 + SP_W * 9 * SP_W,     // [64][9][64]
  SF_N = SF_OFF_F2 + SP_W * 9 * SP_W
};
static_assert(SP_OFF_W2 % 8 == 0 && SP_OFF_W3 % 8 == 0 && SP_OFF_W4 % 8 == 0, "16-byte aligned bf16 weights");

// the network's device state: parameters, Adam moments, activations and
// gradients of up to maxB grids of N1 x N0 cells, reduction scratch
struct SurrogateNet {
  int N0 = 0, N1 = 0, C = 0, maxB = 0;
  int64_t Pmax = 0;
  int num_sms = 148;
  float *p32 = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
  __nv_bfloat16 *w16 = nullptr, *f16 = nullptr;
  __nv_bfloat16 *xin = nullptr, *a1 = nullptr, *a2 = nullptr, *a3 = nullptr;
  __nv_bfloat16 *dzA = nullptr, *dzB = nullptr, *dz4 = nullptr;
  float* y = nullptr;
  float *part = nullptr, *partb = nullptr;
  double *lpart = nullptr, *loss = nullptr, *loss_h = nullptr;
  double oscale = 1.0;
  uint32_t* status = nullptr;  // device status word of the standalone calls
  cudaStream_t stream = nullptr;
  bool tc = false;     // 64->64 layers of inference on tcgen05
  bool tc_ok = false;  // the tcgen05 kernel and the TMA encoder are available
  int64_t tc_launches = 0;
  std::string err;
};
struct Session;

// a network input value v = 10 (b n - 0.25) as the bf16 pair (hi, lo):
// hi = bf16(v), lo = bf16(v - hi)
__device__ __forceinline__ void sur_hi_lo(double v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn((float)v);
  lo = __float2bfloat16_rn((float)(v - (double)__bfloat162float(hi)));
}

// tcgen05 implicit-GEMM 3x3 convolutions of inference (mcpm_surrogate_tc.cu):
// 64 -> 64 and 16 -> 64 with bias and ReLU, and the 64 -> 16 output layer
// (its four used outputs into pcell's kick coefficients, or as y [P][4]);
// each returns its launches, -1 when a tensor map was refused
int tc_setup();
int tc_conv64_relu(const __nv_bfloat16* x, const __nv_bfloat16* w, const float* bias, __nv_bfloat16* out, int N0,
                   int N1, int P, int num_sms, uint32_t* status, cudaStream_t st);
int tc_conv16_relu(const __nv_bfloat16* x, const __nv_bfloat16* w, const float* bias, __nv_bfloat16* out, int N0,
                   int N1, int P, int num_sms, uint32_t* status, cudaStream_t st);
int tc_conv_out(const __nv_bfloat16* x, const __nv_bfloat16* w, const float* bias, float* y, float* pcell, float g1,
                float g2, float oscale, int N0, int N1, int P, int num_sms, uint32_t* status, cudaStream_t st);
// the backward data gradient cin -> 64 (cin = 16 or 64; the transposed and
// flipped weights), gated by the forward activation's sign (training)
int tc_conv_mask(int cin, const __nv_bfloat16* x, const __nv_bfloat16* w, const __nv_bfloat16* mask,
                 __nv_bfloat16* out, int N0, int N1, int P, int num_sms, uint32_t* status, cudaStream_t st);

// session-side launchers (mcpm_surrogate.cu); each returns its launches
int sur_forward_kick(Session& s, const double* nnd, const double* ncell);
int sur_judge(Session& s, const double* nnd, const double* ncell);
// the judge in two parts: the network's output for the comparison, then the
// comparison with the plain path's kick in the record (the plain path may
// run on another stream in between)
int sur_judge_forward(Session& s, const double* nnd, const double* ncell);
int sur_judge_compare(Session& s);
int sur_snapshot(Session& s, const double* fld_dev, int K, uint64_t seed, uint32_t snap, int32_t* qc, double* nnd,
                 double* ncell, uint16_t* x, float* y);

}  // namespace mcpm
