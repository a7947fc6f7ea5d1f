// Declarations shared by the learned warm-start kernels (vg_nn_conv.cu, vg_nn.cu).
//
// Tensors are channels-last BF16 ([D][H][W][C], C a multiple of 16); weights
// of a 3x3x3 convolution are [27][Co][Ci] BF16 with tap = (dz+1)*9 + (dy+1)*3 + (dx+1).
#pragma once

#include <cuda_bf16.h>

#include "vg_internal.cuh"

namespace vg {
namespace nn {

// Input of a convolution: x1 (C1 channels), optionally read through a
// nearest-neighbour 2x upsampling (x1 then has dims D/2, H/2, W/2), followed
// by x2 (C2 channels, may be 0) at the output resolution D x H x W.
struct ConvIn {
  const __nv_bfloat16* x1;
  const __nv_bfloat16* x2;
  int C1, C2;
  int up1;
  int D, H, W;
};

// Output: y (BF16) or yf (FP32), Co channels; + bias, then the leaky ReLU
// (v > 0 ? v : slope v) when relu != 0, then, with a mask tensor (same layout
// as the output), a factor mask_slope wherever the mask entry is <= 0 (the
// derivative of that activation, for input gradients).
struct ConvOut {
  __nv_bfloat16* y;
  float* yf;
  const float* bias;
  const __nv_bfloat16* mask;
  int Co;
  int relu;
  float slope;
  float mask_slope;
};

bool conv_shape_ok(int D, int H, int W, int C1, int C2, int Co);
size_t conv3_fwd_smem(int D, int H, int W, int co_t);
vg_status conv3_fwd(Ctx* c, const ConvIn& in, const __nv_bfloat16* wt, const ConvOut& out);
// The tcgen05 form (tiles of 8 x 16 voxels; needs W % 8 == 0, H % 16 == 0, the
// weights of one output-channel group within shared memory, and c->dflag for
// its timeout bit); *handled says whether it ran.
vg_status conv3_fwd_umma(Ctx* c, const ConvIn& in, const __nv_bfloat16* wt, const ConvOut& out, bool* handled);
// dW[27][Co][Ci] += sum over voxels of dY (x) X_tap  (FP32, accumulated atomically)
vg_status conv3_wgrad(Ctx* c, const ConvIn& in, const __nv_bfloat16* dy, int Co, float* dw);

}  // namespace nn
}  // namespace vg
