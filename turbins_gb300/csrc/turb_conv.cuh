// turb_conv.cuh -- BF16 tensor-core 3x3x3 convolutions (k_conv.cu) used by
// the pressure-guess network (k_net.cu).
//
// Activation layout ("channel-blocked"): a tensor of C channels on an
// X x Y x Z voxel grid is stored as [C/8][Z][Y][X][8] BF16, i.e. C/8 planes
// of 16-byte vectors.  A TMA box of 8 x bx x by x bz x kc/8 elements lands in
// shared memory as [kc/8][voxel][8], which is directly a tcgen05 operand:
// K-major (channels = K) for the forward and data-gradient convolutions, and
// MN-major (voxels = K) for the weight gradient.
#pragma once
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

typedef __nv_bfloat16 bf16;

// how one convolution on one grid is tiled
struct ConvPlan {
    int slab;                 // 1: 128-voxel x rows, one halo slab per channel chunk
    int rows;                 // 1: row-ring kernel (cp.async rows, resident weights)
    int kc, nkc;              // channels per K chunk, number of chunks
    int bx, by, bz, nb;       // output tile (nb = bx*by*bz <= 128 voxels)
    int ntx, nty, ntz, ntiles;
    int wres;                 // all weights resident in shared memory
    int sa, sb;               // A / B pipeline stages
    uint32_t abytes, bbytes, astride, bstride, wbytes, a_lbo, smem;
    int ncols;                // TMEM columns (2 accumulators)
};
ConvPlan conv_plan(int X, int Y, int Z, int cin, int cout);

// Epilogue options of a convolution: out = mask?( relu?( acc + bias + skip ) )
// and, for a 16-channel output, an optional 1x1x1 head hout = headw . out + headb
struct ConvEpi {
    const float *bias = nullptr;
    int relu = 0;
    const bf16 *skip = nullptr;
    const bf16 *mask = nullptr;
    bf16 *out = nullptr;
    const float *headw = nullptr;
    const float *headb = nullptr;
    float *hout = nullptr;
};

// Weight packs: W[27][cout][cin] FP32 -> the B operand of the forward
// convolution and of the data-gradient convolution (taps mirrored, cin and
// cout exchanged), in the layout of the kernel each plan selects.
void conv_pack_weights(cudaStream_t s, const float *W, int cin, int cout, const ConvPlan &pf, const ConvPlan &pb,
                       bf16 *wf, bf16 *wd);

// elements of a weight pack buffer for a conv of (cin, cout) on any grid
// (the row kernel's layout pads K to 128-byte rows); buffers start zeroed
inline long long conv_pack_elems(int cin, int cout)
{
    long long std = 27LL * cin * cout;
    long long rows = 3LL * ((3 * cin + 63) / 64) * 3 * cout * 64;
    return std > rows ? std : rows;
}

int conv3_fwd(cudaStream_t s, const bf16 *in, int X, int Y, int Z, int cin, int cout, const bf16 *wpk,
              const ConvEpi &e, int *err, int nsm);
int conv3_wgrad(cudaStream_t s, const bf16 *x, const bf16 *dy, int X, int Y, int Z, int cin, int cout, float *dw,
                int *err, int nsm);
int conv_selftest_umma(int mn_major, int swap, unsigned long long *mismatches);
const char *conv_last_error();
