// denoiser.hpp -- launchers of the denoiser kernels (denoiser_kernels.cu) and the
// network that drives them (denoiser.cpp).  Tensors are [B][D][H][W][C] bf16,
// C a multiple of 16; weights [Cout][27][Cin] bf16 with tap (dz+1)*9+(dy+1)*3+(dx+1).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "engine.hpp"

namespace dxmcg {
namespace nn {

// Input of a convolution: channels [0, ca) from tensor a (at half resolution,
// nearest-upsampled on the fly, when halfA), channels [ca, ca + cb) from b.
struct ConvIn {
    const __nv_bfloat16* a = nullptr;
    int ca = 0;
    int halfA = 0;
    const __nv_bfloat16* b = nullptr;
    int cb = 0;
};

size_t conv3SmemBytes(int nt);
size_t wgradSmemBytes(int nt);
cudaError_t conv3Configure(); // opt the kernels into their shared-memory size (once per device)

// Options of the tcgen05 convolution beyond launchConv3's:
//   list:   device array of output-brick indices (conv3TcBrickDims, x fastest, then y,
//           z, batch) and *listLen, its length, on the device: only those bricks are
//           computed, the others' output is left as it was;
//   pooled: also the 2x2x2 average of the (bf16) output, as launchAvgPool gives it up
//           to the order of the eight additions (D, H, W even);
//   head:   for a 16-channel output, the 1x1x1 head (16 weights, then the bias) in
//           place of the output, exactly as launchHead without a target: headPred[v]
//           = the prediction, headOut[v] = it times headScale (either may be null);
//   handoverPolls: polls of each wait by which one role of the kernel hands work to
//           another before it gives up (0: 2^24); the waits for copies and MMAs already
//           in flight keep the default limit, so a kernel that gives up still returns
//           only after its own asynchronous work has landed.
struct ConvOptions {
    const int* list = nullptr;
    const int* listLen = nullptr;
    __nv_bfloat16* pooled = nullptr;
    const float* head = nullptr;
    float* headPred = nullptr;
    double* headOut = nullptr;
    double headScale = 1.0;
    uint32_t handoverPolls = 0;
};

// tcgen05 (5th-generation tensor core) form of launchConv3 (conv_tc.cu); the same
// arguments and result up to FP32 summation order, plus the optional epilogue work
cudaError_t conv3TcConfigure();
cudaError_t launchConv3Tc(const ConvIn& in, int B, int D, int H, int W, int Cin, const __nv_bfloat16* w,
    const float* bias, int Cout, bool relu, __nv_bfloat16* out, cudaStream_t s, const ConvOptions* ep = nullptr);
cudaError_t conv3TcErrors(unsigned* flags);
// CTAs of the tcgen05 launch for this shape (a grid under one CTA per SM leaves the
// tensor cores of the other SMs idle: the caller then takes launchConv3)
int conv3TcCtas(int B, int D, int H, int W, int Cout);
// the output bricks of the tcgen05 launch for this shape: (x, y, z) voxels per brick
// and the brick counts along x, y, z (per batch item)
void conv3TcBrickDims(int D, int H, int W, int Cout, int brick[3], int count[3]);
// Brick sets of the world path (one byte per brick, bricks x fastest, all on the device;
// the tissue set comes from launchPrepareInput's brick marks):
//   grow:     the marked bricks and their 26 neighbours;
//   map:      bricks of another brick grid (outCount per axis) that a marked brick
//             needs: the union over marked bricks (cx, cy, cz) of the boxes
//             X(cx) x Y(cy) x Z(cz), where `ranges` (device) holds for each output brick
//             index b along x, then y, then z, the range [lo, hi] of input brick indices
//             whose interval holds b; three one-axis passes (tmp1: outCount[0] x
//             inCount[1] x inCount[2] bytes, tmp2: outCount[0] x outCount[1] x
//             inCount[2]);
//   list:     the marked indices in increasing order, and how many (*listLen);
//             launchBrickLists compacts up to kMaxBrickLists masks in one launch.
cudaError_t launchBrickGrow(const uint8_t* active, const int count[3], uint8_t* grown, cudaStream_t s);
cudaError_t launchBrickMap(const uint8_t* in, const int inCount[3], const int outCount[3], const int* ranges,
    uint8_t* out, uint8_t* tmp1, uint8_t* tmp2, cudaStream_t s);
cudaError_t launchBrickList(const uint8_t* mask, int nb, int* list, int* listLen, cudaStream_t s);
constexpr int kMaxBrickLists = 12;
struct BrickListJobs {
    const uint8_t* mask[kMaxBrickLists] = {};
    int* list[kMaxBrickLists] = {};
    int* len[kMaxBrickLists] = {};
    int nb[kMaxBrickLists] = {};
    int n = 0;
    void add(const uint8_t* m, int count, int* l, int* lenOut)
    {
        if (n < kMaxBrickLists) {
            mask[n] = m;
            nb[n] = count;
            list[n] = l;
            len[n] = lenOut;
        }
        ++n; // beyond kMaxBrickLists the launch refuses
    }
};
cudaError_t launchBrickLists(const BrickListJobs& jobs, cudaStream_t s);
// out = act(conv3(in) + bias), act = relu or identity; bias may be null
cudaError_t launchConv3(const ConvIn& in, int B, int D, int H, int W, int Cin, const __nv_bfloat16* w,
    const float* bias, int Cout, bool relu, __nv_bfloat16* out, cudaStream_t s);
// dW[co][t][ci] += sum_v dz[v][co] x[v + off(t)][ci]  (FP32 atomics)
cudaError_t launchWgrad(const ConvIn& in, const __nv_bfloat16* dz, int B, int D, int H, int W, int Cin, int Cout,
    float* dW, cudaStream_t s);
// dz = dy * (y > 0), db += sum over voxels of dz
cudaError_t launchReluBackward(const __nv_bfloat16* dy, const __nv_bfloat16* y, __nv_bfloat16* dz, size_t nvox,
    int C, float* db, cudaStream_t s);
cudaError_t launchAvgPool(const __nv_bfloat16* x, __nv_bfloat16* out, int B, int D, int H, int W, int C,
    cudaStream_t s);
// du (half res) = sum of children of dcat[:, :cu]; de = dcat[:, cu:] + dxNext(parent) / 8 (either may be null)
cudaError_t launchSplitConcatGrad(const __nv_bfloat16* dcat, int cu, int cs, const __nv_bfloat16* dxNext,
    __nv_bfloat16* du, __nv_bfloat16* de, int B, int D, int H, int W, cudaStream_t s);
// head: pred = d . w + b; with a target also the L1 loss sum and the gradients
cudaError_t launchHead(const __nv_bfloat16* d, int C0, const float* hw, size_t nvox, const float* target,
    float* pred, double predScale, double* predOut, __nv_bfloat16* dd, float* dhw, double* lossSum, cudaStream_t s);
cudaError_t launchAdam(float* p, const float* g, float* m, float* v, __nv_bfloat16* pb, size_t n, float lr, float b1,
    float b2, float eps, float c1, float c2, cudaStream_t s);
cudaError_t launchToBf16(const float* p, __nv_bfloat16* pb, size_t n, cudaStream_t s);
cudaError_t launchTransposeWeights(const __nv_bfloat16* w, __nv_bfloat16* wt, int Cout, int Cin, cudaStream_t s);
// Bricks to mark while the input is prepared from a world: active[b] = 1 for each
// brick b holding a voxel whose material is not 0 (bricks of bx, by, bz voxels, cx and
// cy of them along x and y, x fastest; the grid nx voxels along x, ny along y).  The
// caller zeroes `active`.
struct BrickMarks {
    uint8_t* active = nullptr;
    int nx = 1, ny = 1, bx = 1, by = 1, bz = 1, cx = 1, cy = 1;
};
// input channels [log1p(d / s), density, one-hot(material 0..5), 0 x 8] from arrays
// (dose, dens, mat) or from a world (tally, vox, toDose); with a world, optionally
// the brick marks above (fewer than 2^32 voxels)
cudaError_t launchPrepareInput(const float* dose, const float* dens, const uint8_t* mat, const Tally* tally,
    const uint32_t* vox, double toDose, size_t n, float invScale, __nv_bfloat16* out, cudaStream_t s,
    const BrickMarks* marks = nullptr);
// patches outside their volume (or of a volume index out of range) are written as zeros
cudaError_t launchGatherPatches(const __nv_bfloat16* const* inputs, const float* const* targets, const int* dims,
    int nVolumes, const int* origins, int nPatch, int P, __nv_bfloat16* xin, float* tgt, cudaStream_t s);
cudaError_t launchDoseMean(const Tally* tally, const uint32_t* vox, double toDose, size_t n, float rhoMin,
    double* sum, unsigned long long* count, cudaStream_t s);

// a world's dose through the network (denoiser.cpp); dims nx, ny, nz (x fastest)
int denoiseWorld(dxmcg_denoiser* d, int device, const Tally* tally, const uint32_t* vox, int nx, int ny, int nz,
    double toDose, double scale, double* hostOut, double* scaleUsed, cudaStream_t s);

} // namespace nn
} // namespace dxmcg
