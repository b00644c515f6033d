// denoiser.cpp -- the dose denoiser network on the GPU: parameters, activation
// buffers, forward, backward and Adam, and the C ABI (include/dxmcg.h).  Every
// tensor operation is a kernel of denoiser_kernels.cu.  No counterpart in the
// reference.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "../../include/dxmcg.h"
#include "denoiser.hpp"
#include "devbuf.hpp"

using namespace dxmcg;
using bf16 = __nv_bfloat16;

#define NN_CUDA(call)                                                                                               \
    do {                                                                                                            \
        const cudaError_t e_ = (call);                                                                              \
        if (e_ != cudaSuccess)                                                                                      \
            return reportError(DXMCG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));                \
    } while (0)

struct dxmcg_denoiser {
    struct Layer {
        int cin, cout;
        size_t w, b, wt; // offsets: weights and bias in the parameter vector, weights in the transposed copy
    };
    int device = 0;
    int L = 0;
    int ch[5] {};
    std::vector<Layer> layers;
    size_t head = 0, nParams = 0, nWt = 0;
    DevBuf<float> p, g, m, v;
    DevBuf<bf16> pb, wt;
    long step = 0;
    bool configured = false;
    bool tensorCores = true;  // tcgen05 convolutions (else warp-level mma.sync)
    bool tcEverywhere = false; // tcgen05 even where the grid has fewer bricks than SMs
    int sms = 1;              // streaming multiprocessors of the device
    uint32_t waitPolls = 0;   // hand-over wait limit of the tcgen05 convolution (0: default)

    // activations and gradients of the current shape, per level
    int B = 0, D = 0, H = 0, W = 0;
    std::vector<DevBuf<bf16>> x, ea, eb, da, db, gx, gea, geb, gda, gdb, dcat;
    DevBuf<bf16> dz;
    DevBuf<float> pred;
    DevBuf<double> loss;
    // world path: input channels, denoised dose and the normalisation sums, kept
    // between calls (the input of a 512x512x400 world is 3.4 GB)
    DevBuf<bf16> worldInput;
    DevBuf<double> worldOut, meanSum;
    // world path: brick masks and lists of the restricted layers (level 0: tissue and
    // tissue grown by one; the decoders of levels 1-2 and the encoders of levels 0-2:
    // the bricks that the tissue bricks need), two scratch masks and the brick ranges
    // that map the tissue bricks onto those grids
    DevBuf<uint8_t> mask0[2], mask1[2], mask2[2], maskEnc[3], maskTmp[2];
    DevBuf<int> list0[2], list1[2], list2[2], listEnc[3], listLens, encRanges;
    std::vector<int> encRangesHost;
    DevBuf<unsigned long long> meanCount;

    int encA(int l) const { return 2 * l; }
    int encB(int l) const { return 2 * l + 1; }
    int decA(int l) const { return 2 * L + 2 * (L - 2 - l); }
    int decB(int l) const { return decA(l) + 1; }
    size_t nvox(int l) const { return static_cast<size_t>(B) * (D >> l) * (H >> l) * (W >> l); }
};

namespace {

int fail(int code, const std::string& msg) { return reportError(code, msg); }

int ensureShape(dxmcg_denoiser* d, int B, int D, int H, int W)
{
    const int f = 1 << (d->L - 1);
    if (B < 1 || D < f || H < f || W < f || D % f || H % f || W % f)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser: dims must be positive multiples of 2^(levels-1)");
    if (d->B == B && d->D == D && d->H == H && d->W == W)
        return DXMCG_OK;
    d->B = B;
    d->D = D;
    d->H = H;
    d->W = W;
    const int L = d->L;
    for (auto* vec : { &d->x, &d->ea, &d->eb, &d->da, &d->db, &d->gx, &d->gea, &d->geb, &d->gda, &d->gdb,
             &d->dcat }) {
        vec->clear();
        vec->resize(L);
    }
    size_t dzMax = 0;
    for (int l = 0; l < L; ++l) {
        const size_t n = d->nvox(l);
        const size_t c = d->ch[l];
        if (l > 0) {
            NN_CUDA(d->x[l].reserve(n * d->ch[l - 1]));
            NN_CUDA(d->gx[l].reserve(n * d->ch[l - 1]));
        }
        NN_CUDA(d->ea[l].reserve(n * c));
        NN_CUDA(d->eb[l].reserve(n * c));
        NN_CUDA(d->gea[l].reserve(n * c));
        NN_CUDA(d->geb[l].reserve(n * c));
        if (l < L - 1) {
            NN_CUDA(d->da[l].reserve(n * c));
            NN_CUDA(d->db[l].reserve(n * c));
            NN_CUDA(d->gda[l].reserve(n * c));
            NN_CUDA(d->gdb[l].reserve(n * c));
            NN_CUDA(d->dcat[l].reserve(n * (c + d->ch[l + 1])));
        }
        dzMax = std::max(dzMax, n * c);
    }
    NN_CUDA(d->dz.reserve(dzMax));
    NN_CUDA(d->pred.reserve(d->nvox(0)));
    NN_CUDA(d->loss.reserve(1));
    return DXMCG_OK;
}

int refreshWeights(dxmcg_denoiser* d, cudaStream_t s)
{
    for (const auto& ly : d->layers)
        NN_CUDA(nn::launchTransposeWeights(d->pb.p + ly.w, d->wt.p + ly.wt, ly.cout, ly.cin, s));
    return DXMCG_OK;
}

// tcgen05 for a convolution unless its grid would leave SMs without a CTA (or always,
// when asked for with conv_path 1)
bool useTensorCores(const dxmcg_denoiser* d, int D, int H, int W, int Cout)
{
    return d->tensorCores && (d->tcEverywhere || nn::conv3TcCtas(d->B, D, H, W, Cout) >= d->sms);
}

// conv + bias + ReLU of layer k at level l; on the tcgen05 path the epilogue also does
// the work of `ep` (*fused is set then; the caller runs the separate kernels otherwise)
int conv(dxmcg_denoiser* d, int k, const nn::ConvIn& in, int l, bf16* out, cudaStream_t s,
    const nn::ConvOptions* ep = nullptr, bool* fused = nullptr)
{
    const auto& ly = d->layers[k];
    const int Dl = d->D >> l, Hl = d->H >> l, Wl = d->W >> l;
    const bool tc = useTensorCores(d, Dl, Hl, Wl, ly.cout);
    if (fused)
        *fused = tc && ep;
    if (tc) {
        nn::ConvOptions o = ep ? *ep : nn::ConvOptions {};
        o.handoverPolls = d->waitPolls;
        NN_CUDA(nn::launchConv3Tc(in, d->B, Dl, Hl, Wl, ly.cin, d->pb.p + ly.w, d->p.p + ly.b, ly.cout, true, out, s,
            &o));
    }
    else
        NN_CUDA(nn::launchConv3(in, d->B, Dl, Hl, Wl, ly.cin, d->pb.p + ly.w, d->p.p + ly.b, ly.cout, true, out, s));
    return DXMCG_OK;
}

// DXMCG_OK unless a tcgen05 convolution gave up waiting for its tensor-core work
// (the kernel then skipped its output); call after a synchronisation
int tensorCoreStatus(dxmcg_denoiser* d)
{
    if (!d->tensorCores)
        return DXMCG_OK;
    unsigned flags = 0;
    NN_CUDA(nn::conv3TcErrors(&flags));
    if (flags)
        return fail(DXMCG_ERR_DEVICE, "denoiser: a tensor-core convolution timed out waiting for its MMAs");
    return DXMCG_OK;
}

nn::ConvIn plain(const bf16* t, int c)
{
    nn::ConvIn in;
    in.a = t;
    in.ca = c;
    return in;
}

// input of decoder level l: upsample(d_{l+1}) ++ e_lb
nn::ConvIn decIn(dxmcg_denoiser* d, int l)
{
    nn::ConvIn in;
    in.a = l + 1 < d->L - 1 ? d->db[l + 1].p : d->eb[d->L - 1].p;
    in.ca = d->ch[l + 1];
    in.halfA = 1;
    in.b = d->eb[l].p;
    in.cb = d->ch[l];
    return in;
}

nn::ConvIn encIn(dxmcg_denoiser* d, int l, const bf16* input)
{
    return l == 0 ? plain(input, 16) : plain(d->x[l].p, d->ch[l - 1]);
}

const bf16* finalActivation(dxmcg_denoiser* d) { return d->L > 1 ? d->db[0].p : d->eb[0].p; }

// Span of level-0 voxels [lo, hi] along one axis.
struct Span {
    int lo, hi;
};

Span widen(Span s, int r) { return { s.lo - r, s.hi + r }; }

int floorHalf(int a) { return a >= 0 ? a / 2 : -((1 - a) / 2); }

// What a span describes (level-l voxels of one tensor, along one axis): the output
// of the encoder of level l widened by one voxel (its two convolutions: the second
// reads the first with a one-voxel halo), or the output of the second or the first
// convolution of the decoder of level l.
enum SpanKind { kEncoderPair, kDecoderSecond, kDecoderFirst };
struct SpanTarget {
    SpanKind kind;
    int level;
};

void fold(Span& acc, Span s) { acc = { std::min(acc.lo, s.lo), std::max(acc.hi, s.hi) }; }

// Fold into `acc` the voxels of the target on which the encoder output (second
// convolution) of level l on span s depends: two 3-tap convolutions per level, and the
// 2x2x2 average pooling between levels (voxel q of level l reads voxels 2q and 2q + 1
// of level l - 1).  An encoder output depends on no decoder output, and on no encoder
// deeper than itself.
void encoderNeeds(int l, SpanTarget t, Span s, Span& acc)
{
    if (t.kind != kEncoderPair || l < t.level)
        return;
    if (l == t.level) {
        fold(acc, s);
        return;
    }
    const Span x = widen(s, 2);
    encoderNeeds(l - 1, t, { 2 * x.lo, 2 * x.hi + 1 }, acc);
}

// The same for the decoder output of level l (l < L - 1) on span s: its second
// convolution reads the first with a one-voxel halo, and the first reads the skip
// input (the encoder output of level l) and the nearest upsampling of level l + 1
// (voxel v reads voxel floor(v / 2)) with another.
void decoderNeeds(int L, int l, SpanTarget t, Span s, Span& acc)
{
    if (t.kind == kDecoderSecond && l == t.level)
        fold(acc, s);
    if (t.kind == kDecoderFirst && l == t.level)
        fold(acc, widen(s, 1));
    const Span in = widen(s, 2);
    encoderNeeds(l, t, in, acc);
    const Span up = { floorHalf(in.lo), floorHalf(in.hi) };
    if (l + 1 == L - 1)
        encoderNeeds(L - 1, t, up, acc);
    else
        decoderNeeds(L, l + 1, t, up, acc);
}

// Along one axis: the voxels of the target that the network's outputs on level-0
// voxels [p0, p1] depend on (empty: lo > hi).
Span networkSpan(int L, SpanTarget t, int p0, int p1)
{
    Span acc { INT_MAX, INT_MIN };
    for (int p = p0; p <= p1; ++p)
        decoderNeeds(L, 0, t, { p, p }, acc);
    if (acc.lo > acc.hi)
        return acc;
    return t.kind == kEncoderPair ? widen(acc, 1) : acc;
}

// For each brick b of the target's grid along one axis (nl bricks of bl voxels over
// diml voxels): the range [out[2b], out[2b + 1]] of level-0 bricks (n0 of b0 voxels
// over dim0) whose outputs need it; an empty range where none does.
void brickRanges(int L, SpanTarget t, int dim0, int b0, int n0, int diml, int bl, int nl, int* out)
{
    for (int b = 0; b < nl; ++b) {
        out[2 * b] = n0;
        out[2 * b + 1] = -1;
    }
    for (int c = 0; c < n0; ++c) {
        const int p0 = c * b0, p1 = std::min(p0 + b0, dim0) - 1;
        const Span sp = networkSpan(L, t, p0, p1);
        const int lo = std::max(0, sp.lo), hi = std::min(diml - 1, sp.hi);
        for (int b = lo / bl; lo <= hi && b <= hi / bl && b < nl; ++b) {
            out[2 * b] = std::min(out[2 * b], c);
            out[2 * b + 1] = std::max(out[2 * b + 1], c);
        }
    }
}

// Forward pass.  The encoder's pooling is fused into the second convolution of each
// level where that runs on tcgen05.  With `pred` or `predOut` (inference) the 1x1x1
// head follows: fused into the last convolution (whose output is then not stored)
// where it can be, else by headKernel; pred = prediction, predOut = prediction *
// predScale.  `sparse` (inference, head fused) restricts the last convolution to the
// bricks sparse->last marks and the one before it to sparse->before.
struct Sparse {
    const int* last = nullptr; // brick list of the last convolution, its length at lastLen
    const int* lastLen = nullptr;
    const int* before = nullptr; // and of the one before
    const int* beforeLen = nullptr;
    const int* dec1b = nullptr; // level-1 decoder (null: dense)
    const int* dec1bLen = nullptr;
    const int* dec1a = nullptr;
    const int* dec1aLen = nullptr;
    const int* dec2b = nullptr; // level-2 decoder (null: dense)
    const int* dec2bLen = nullptr;
    const int* dec2a = nullptr;
    const int* dec2aLen = nullptr;
    const int* enc[3] = {}; // both encoder convolutions of levels 0-2 (null: dense)
    const int* encLen[3] = {};
};

int forward(dxmcg_denoiser* d, const bf16* input, cudaStream_t s, float* pred = nullptr,
    double* predOut = nullptr, double predScale = 1.0, const Sparse* sparse = nullptr)
{
    int rc;
    const bool wantHead = pred || predOut;
    nn::ConvOptions headEp;
    headEp.head = d->p.p + d->head;
    headEp.headPred = pred;
    headEp.headOut = predOut;
    headEp.headScale = predScale;
    if (sparse) {
        headEp.list = sparse->last;
        headEp.listLen = sparse->lastLen;
    }
    nn::ConvOptions beforeEp;
    if (sparse) {
        beforeEp.list = sparse->before;
        beforeEp.listLen = sparse->beforeLen;
    }
    const bool headFusable = wantHead && d->ch[0] == 16;
    bool headDone = false;
    for (int l = 0; l < d->L; ++l) {
        const bool last = d->L == 1; // encB(0) is the final convolution of a one-level net
        nn::ConvOptions encEp;
        const bool sparseEnc = sparse && l < 3 && l < d->L - 1 && sparse->enc[l];
        if (sparseEnc) {
            encEp.list = sparse->enc[l];
            encEp.listLen = sparse->encLen[l];
        }
        const nn::ConvOptions* epA = last && sparse ? &beforeEp : (sparseEnc ? &encEp : nullptr);
        if ((rc = conv(d, d->encA(l), encIn(d, l, input), l, d->ea[l].p, s, epA)) != DXMCG_OK)
            return rc;
        nn::ConvOptions ep;
        if (l < d->L - 1) {
            ep.pooled = d->x[l + 1].p;
            ep.list = encEp.list;
            ep.listLen = encEp.listLen;
        } else if (last && headFusable)
            ep = headEp;
        bool fused = false;
        const bool withEp = ep.pooled || ep.head;
        if ((rc = conv(d, d->encB(l), plain(d->ea[l].p, d->ch[l]), l, d->eb[l].p, s, withEp ? &ep : nullptr,
                 &fused))
            != DXMCG_OK)
            return rc;
        if (l < d->L - 1 && !fused)
            NN_CUDA(nn::launchAvgPool(d->eb[l].p, d->x[l + 1].p, d->B, d->D >> l, d->H >> l, d->W >> l, d->ch[l], s));
        if (last && ep.head)
            headDone = fused;
    }
    nn::ConvOptions dec1aEp, dec1bEp, dec2aEp, dec2bEp;
    if (sparse && sparse->dec1a) {
        dec1aEp.list = sparse->dec1a;
        dec1aEp.listLen = sparse->dec1aLen;
        dec1bEp.list = sparse->dec1b;
        dec1bEp.listLen = sparse->dec1bLen;
    }
    if (sparse && sparse->dec2a) {
        dec2aEp.list = sparse->dec2a;
        dec2aEp.listLen = sparse->dec2aLen;
        dec2bEp.list = sparse->dec2b;
        dec2bEp.listLen = sparse->dec2bLen;
    }
    const bool sparse1 = sparse && sparse->dec1a;
    const bool sparse2 = sparse && sparse->dec2a;
    for (int l = d->L - 2; l >= 0; --l) {
        const nn::ConvOptions* epA = l == 0 && sparse
            ? &beforeEp
            : (l == 1 && sparse1 ? &dec1aEp : (l == 2 && sparse2 ? &dec2aEp : nullptr));
        if ((rc = conv(d, d->decA(l), decIn(d, l), l, d->da[l].p, s, epA)) != DXMCG_OK)
            return rc;
        const bool withHead = l == 0 && headFusable;
        bool fused = false;
        const nn::ConvOptions* epB
            = withHead ? &headEp : (l == 1 && sparse1 ? &dec1bEp : (l == 2 && sparse2 ? &dec2bEp : nullptr));
        if ((rc = conv(d, d->decB(l), plain(d->da[l].p, d->ch[l]), l, d->db[l].p, s, epB, &fused)) != DXMCG_OK)
            return rc;
        if (withHead)
            headDone = fused;
    }
    if (wantHead && !headDone)
        NN_CUDA(nn::launchHead(finalActivation(d), d->ch[0], d->p.p + d->head, d->nvox(0), nullptr, pred, predScale,
            predOut, nullptr, nullptr, nullptr, s));
    return DXMCG_OK;
}

// relu backward + weight/bias gradients, and the input gradient when dxOut
int layerBack(dxmcg_denoiser* d, int k, const nn::ConvIn& xin, const bf16* y, const bf16* dy, bf16* dxOut, int l,
    cudaStream_t s)
{
    const auto& ly = d->layers[k];
    const int Dl = d->D >> l, Hl = d->H >> l, Wl = d->W >> l;
    NN_CUDA(nn::launchReluBackward(dy, y, d->dz.p, d->nvox(l), ly.cout, d->g.p + ly.b, s));
    NN_CUDA(nn::launchWgrad(xin, d->dz.p, d->B, Dl, Hl, Wl, ly.cin, ly.cout, d->g.p + ly.w, s));
    if (dxOut) {
        if (useTensorCores(d, Dl, Hl, Wl, ly.cin)) {
            nn::ConvOptions o;
            o.handoverPolls = d->waitPolls;
            NN_CUDA(nn::launchConv3Tc(plain(d->dz.p, ly.cout), d->B, Dl, Hl, Wl, ly.cout, d->wt.p + ly.wt, nullptr,
                ly.cin, false, dxOut, s, &o));
        }
        else
            NN_CUDA(nn::launchConv3(plain(d->dz.p, ly.cout), d->B, Dl, Hl, Wl, ly.cout, d->wt.p + ly.wt, nullptr,
                ly.cin, false, dxOut, s));
    }
    return DXMCG_OK;
}

int backward(dxmcg_denoiser* d, const bf16* input, const float* target, cudaStream_t s)
{
    NN_CUDA(cudaMemsetAsync(d->g.p, 0, d->nParams * sizeof(float), s));
    NN_CUDA(cudaMemsetAsync(d->loss.p, 0, sizeof(double), s));
    const int L = d->L;
    bf16* gFinal = L > 1 ? d->gdb[0].p : d->geb[0].p;
    NN_CUDA(nn::launchHead(finalActivation(d), d->ch[0], d->p.p + d->head, d->nvox(0), target, d->pred.p, 1.0,
        nullptr, gFinal, d->g.p + d->head, d->loss.p, s));
    int rc;
    // decoder, from the head towards the bottleneck
    for (int l = 0; l < L - 1; ++l) {
        if ((rc = layerBack(d, d->decB(l), plain(d->da[l].p, d->ch[l]), d->db[l].p, d->gdb[l].p, d->gda[l].p, l, s))
            != DXMCG_OK)
            return rc;
        if ((rc = layerBack(d, d->decA(l), decIn(d, l), d->da[l].p, d->gda[l].p, d->dcat[l].p, l, s)) != DXMCG_OK)
            return rc;
        bf16* du = l + 1 < L - 1 ? d->gdb[l + 1].p : d->geb[L - 1].p;
        NN_CUDA(nn::launchSplitConcatGrad(d->dcat[l].p, d->ch[l + 1], d->ch[l], nullptr, du, nullptr, d->B,
            d->D >> l, d->H >> l, d->W >> l, s));
    }
    // encoder, from the bottleneck down
    for (int l = L - 1; l >= 0; --l) {
        if (l < L - 1)
            NN_CUDA(nn::launchSplitConcatGrad(d->dcat[l].p, d->ch[l + 1], d->ch[l], d->gx[l + 1].p, nullptr,
                d->geb[l].p, d->B, d->D >> l, d->H >> l, d->W >> l, s));
        if ((rc = layerBack(d, d->encB(l), plain(d->ea[l].p, d->ch[l]), d->eb[l].p, d->geb[l].p, d->gea[l].p, l, s))
            != DXMCG_OK)
            return rc;
        if ((rc = layerBack(d, d->encA(l), encIn(d, l, input), d->ea[l].p, d->gea[l].p, l > 0 ? d->gx[l].p : nullptr,
                 l, s))
            != DXMCG_OK)
            return rc;
    }
    return DXMCG_OK;
}

int checkNet(const dxmcg_denoiser* d)
{
    if (!d)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser: null handle");
    return cudaSetDevice(d->device) == cudaSuccess ? DXMCG_OK : fail(DXMCG_ERR_CUDA, "denoiser: cudaSetDevice");
}

} // namespace

namespace dxmcg {
namespace nn {
    // the world path (capi.cpp): input from a tally, forward, dose = pred * scale
    int denoiseWorld(dxmcg_denoiser* d, int device, const Tally* tally, const uint32_t* vox, int nx, int ny, int nz,
        double toDose, double scale, double* hostOut, double* scaleUsed, cudaStream_t s)
    {
        int rc = checkNet(d);
        if (rc != DXMCG_OK)
            return rc;
        if (d->device != device)
            return fail(DXMCG_ERR_ARGUMENT, "world_denoise: the denoiser and the world are on different devices");
        if ((rc = ensureShape(d, 1, nz, ny, nx)) != DXMCG_OK)
            return rc;
        const size_t n = static_cast<size_t>(nx) * ny * nz;
        if (!(scale > 0.0)) {
            NN_CUDA(d->meanSum.reserve(1));
            NN_CUDA(d->meanCount.reserve(1));
            NN_CUDA(cudaMemsetAsync(d->meanSum.p, 0, sizeof(double), s));
            NN_CUDA(cudaMemsetAsync(d->meanCount.p, 0, sizeof(unsigned long long), s));
            NN_CUDA(launchDoseMean(tally, vox, toDose, n, 0.2f, d->meanSum.p, d->meanCount.p, s));
            double hs = 0;
            unsigned long long hc = 0;
            NN_CUDA(cudaMemcpyAsync(&hs, d->meanSum.p, sizeof(double), cudaMemcpyDeviceToHost, s));
            NN_CUDA(cudaMemcpyAsync(&hc, d->meanCount.p, sizeof(hc), cudaMemcpyDeviceToHost, s));
            NN_CUDA(cudaStreamSynchronize(s));
            scale = hc ? hs / static_cast<double>(hc) : 0.0;
            if (!(scale > 0.0))
                return fail(DXMCG_ERR_STATE, "world_denoise: no dose above 0.2 g/cm3 to normalise by");
        }
        if (scaleUsed)
            *scaleUsed = scale;
        NN_CUDA(d->worldInput.reserve(n * 16));
        NN_CUDA(d->worldOut.reserve(n));
        // The readout deletes the dose of air (material 0).  Where the last two
        // convolutions run on tcgen05 with the head fused, the last one computes only
        // bricks holding a non-air voxel and the one before only those and their
        // neighbours (the last one's halo); the dose of the other voxels is 0.  Every
        // voxel of those bricks gets the same value as the dense pass.
        // The decoders of levels 1 and 2 and the encoders of levels 0-2 run on the bricks
        // of their grids that a tissue brick's outputs need: along each axis, the span of
        // that layer's outputs on which the outputs of a level-0 brick depend (every path
        // through the network, at that brick's alignment to the pooling grids; for an
        // encoder, plus its first convolution's halo).  Every value a tissue brick's
        // output depends on is computed as in the dense pass; what the other bricks hold
        // (stale values from earlier calls) reaches only outputs of bricks outside those
        // sets, which the readout does not use.
        // The input pass marks the tissue bricks; every brick list comes from one launch.
        Sparse sp;
        const bool sparse = d->ch[0] == 16 && useTensorCores(d, nz, ny, nx, d->ch[0]);
        int brick[3] = { 1, 1, 1 }, count[3] = { 1, 1, 1 };
        size_t nb = 0;
        BrickMarks marks;
        if (sparse) {
            conv3TcBrickDims(nz, ny, nx, d->ch[0], brick, count);
            nb = static_cast<size_t>(count[0]) * count[1] * count[2];
            for (auto& m : d->mask0)
                NN_CUDA(m.reserve(nb));
            NN_CUDA(cudaMemsetAsync(d->mask0[0].p, 0, nb, s));
            marks.active = d->mask0[0].p;
            marks.nx = nx;
            marks.ny = ny;
            marks.bx = brick[0];
            marks.by = brick[1];
            marks.bz = brick[2];
            marks.cx = count[0];
            marks.cy = count[1];
        }
        NN_CUDA(launchPrepareInput(nullptr, nullptr, nullptr, tally, vox, toDose, n, static_cast<float>(1.0 / scale),
            d->worldInput.p, s, sparse ? &marks : nullptr));
        if (sparse) {
            for (auto& l : d->list0)
                NN_CUDA(l.reserve(nb));
            NN_CUDA(d->listLens.reserve(9));
            BrickListJobs lists;
            NN_CUDA(launchBrickGrow(d->mask0[0].p, count, d->mask0[1].p, s));
            lists.add(d->mask0[0].p, static_cast<int>(nb), d->list0[0].p, d->listLens.p);
            lists.add(d->mask0[1].p, static_cast<int>(nb), d->list0[1].p, d->listLens.p + 1);
            NN_CUDA(cudaMemsetAsync(d->worldOut.p, 0, n * sizeof(double), s));
            sp.last = d->list0[0].p;
            sp.lastLen = d->listLens.p;
            sp.before = d->list0[1].p;
            sp.beforeLen = d->listLens.p + 1;
            // The encoders of levels 0 .. min(2, L - 2) and the decoders of levels 1 and 2
            // that run on tcgen05: the bricks of their grids that some tissue brick's
            // outputs need, as the union over the tissue bricks of per-axis ranges.
            struct SetSpec {
                SpanTarget t;
                DevBuf<uint8_t>* mask;
                DevBuf<int>* list;
                int lenIndex;
                const int** spList;
                const int** spLen;
                int bl[3], cl[3];
            };
            std::vector<SetSpec> specs;
            const auto tc = [&](int l) { return useTensorCores(d, nz >> l, ny >> l, nx >> l, d->ch[l]); };
            for (int lt = 0; lt < 3 && lt <= d->L - 2 && tc(lt); ++lt)
                specs.push_back({ { kEncoderPair, lt }, &d->maskEnc[lt], &d->listEnc[lt], 4 + lt, &sp.enc[lt],
                    &sp.encLen[lt], {}, {} });
            if (d->L >= 3 && tc(1)) {
                specs.push_back({ { kDecoderSecond, 1 }, &d->mask1[0], &d->list1[0], 2, &sp.dec1b, &sp.dec1bLen, {},
                    {} });
                specs.push_back({ { kDecoderFirst, 1 }, &d->mask1[1], &d->list1[1], 3, &sp.dec1a, &sp.dec1aLen, {},
                    {} });
                if (d->L >= 4 && tc(2)) {
                    specs.push_back({ { kDecoderSecond, 2 }, &d->mask2[0], &d->list2[0], 7, &sp.dec2b, &sp.dec2bLen,
                        {}, {} });
                    specs.push_back({ { kDecoderFirst, 2 }, &d->mask2[1], &d->list2[1], 8, &sp.dec2a, &sp.dec2aLen,
                        {}, {} });
                }
            }
            const int dim0[3] = { nx, ny, nz };
            size_t nRanges = 0, tmp1 = 1, tmp2 = 1;
            for (auto& sc : specs) {
                const int l = sc.t.level;
                conv3TcBrickDims(nz >> l, ny >> l, nx >> l, d->ch[l], sc.bl, sc.cl);
                nRanges += 2 * static_cast<size_t>(sc.cl[0] + sc.cl[1] + sc.cl[2]);
                tmp1 = std::max(tmp1, static_cast<size_t>(sc.cl[0]) * count[1] * count[2]);
                tmp2 = std::max(tmp2, static_cast<size_t>(sc.cl[0]) * sc.cl[1] * count[2]);
            }
            if (!specs.empty()) {
                d->encRangesHost.assign(nRanges, 0);
                size_t off = 0;
                for (auto& sc : specs)
                    for (int a = 0; a < 3; ++a) {
                        brickRanges(d->L, sc.t, dim0[a], brick[a], count[a], dim0[a] >> sc.t.level, sc.bl[a],
                            sc.cl[a], d->encRangesHost.data() + off);
                        off += 2 * static_cast<size_t>(sc.cl[a]);
                    }
                NN_CUDA(d->encRanges.reserve(nRanges));
                NN_CUDA(cudaMemcpyAsync(d->encRanges.p, d->encRangesHost.data(), nRanges * sizeof(int),
                    cudaMemcpyHostToDevice, s));
                NN_CUDA(d->maskTmp[0].reserve(tmp1));
                NN_CUDA(d->maskTmp[1].reserve(tmp2));
                off = 0;
                for (auto& sc : specs) {
                    const size_t nbl = static_cast<size_t>(sc.cl[0]) * sc.cl[1] * sc.cl[2];
                    NN_CUDA(sc.mask->reserve(nbl));
                    NN_CUDA(sc.list->reserve(nbl));
                    NN_CUDA(launchBrickMap(d->mask0[0].p, count, sc.cl, d->encRanges.p + off, sc.mask->p,
                        d->maskTmp[0].p, d->maskTmp[1].p, s));
                    off += 2 * static_cast<size_t>(sc.cl[0] + sc.cl[1] + sc.cl[2]);
                    lists.add(sc.mask->p, static_cast<int>(nbl), sc.list->p, d->listLens.p + sc.lenIndex);
                    *sc.spList = sc.list->p;
                    *sc.spLen = d->listLens.p + sc.lenIndex;
                }
            }
            NN_CUDA(launchBrickLists(lists, s));
        }
        if ((rc = forward(d, d->worldInput.p, s, nullptr, d->worldOut.p, scale, sparse ? &sp : nullptr)) != DXMCG_OK)
            return rc;
        if (hostOut)
            NN_CUDA(cudaMemcpyAsync(hostOut, d->worldOut.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
        NN_CUDA(cudaStreamSynchronize(s));
        return tensorCoreStatus(d);
    }
} // namespace nn
} // namespace dxmcg

extern "C" {

DXMCG_API int dxmcg_denoiser_create(const dxmcg_denoiser_config* c, dxmcg_denoiser** out)
{
    if (!out || !c)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_create: null argument");
    *out = nullptr;
    if (c->levels < 1 || c->levels > 5)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_create: levels must be 1..5");
    for (int l = 0; l < c->levels; ++l)
        if (c->channels[l] < 16 || c->channels[l] % 16 || c->channels[l] > 256)
            return fail(DXMCG_ERR_ARGUMENT, "denoiser_create: channels must be multiples of 16 up to 256");
    if (c->channels[0] != 16 && c->channels[0] != 32)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_create: channels[0] must be 16 or 32");
    if (c->conv_path < 0 || c->conv_path > 2)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_create: conv_path must be 0, 1 or 2");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1)
        return fail(DXMCG_ERR_NO_DEVICE, "denoiser_create: no CUDA device");
    auto d = std::make_unique<dxmcg_denoiser>();
    cudaGetDevice(&d->device);
    d->L = c->levels;
    d->tensorCores = c->conv_path != 2;
    d->tcEverywhere = c->conv_path == 1;
    if (cudaDeviceGetAttribute(&d->sms, cudaDevAttrMultiProcessorCount, d->device) != cudaSuccess || d->sms < 1)
        d->sms = 1;
    for (int l = 0; l < d->L; ++l)
        d->ch[l] = c->channels[l];
    std::vector<std::pair<int, int>> shapes; // (cin, cout) in layer order
    int prev = 16;
    for (int l = 0; l < d->L; ++l) {
        shapes.push_back({ prev, d->ch[l] });
        shapes.push_back({ d->ch[l], d->ch[l] });
        prev = d->ch[l];
    }
    for (int l = d->L - 2; l >= 0; --l) {
        shapes.push_back({ d->ch[l + 1] + d->ch[l], d->ch[l] });
        shapes.push_back({ d->ch[l], d->ch[l] });
    }
    size_t o = 0, ot = 0;
    for (auto [ci, co] : shapes) {
        dxmcg_denoiser::Layer ly { ci, co, o, o + static_cast<size_t>(co) * 27 * ci, ot };
        d->layers.push_back(ly);
        o += static_cast<size_t>(co) * 27 * ci + co;
        ot += static_cast<size_t>(co) * 27 * ci;
    }
    d->head = o;
    d->nParams = o + d->ch[0] + 1;
    d->nWt = ot;
    // He-normal initialisation on the host (std::normal_distribution, seeded)
    std::vector<float> h(d->nParams, 0.0f);
    std::mt19937_64 rng(c->seed);
    for (const auto& ly : d->layers) {
        std::normal_distribution<double> nd(0.0, std::sqrt(2.0 / (27.0 * ly.cin)));
        for (size_t i = ly.w; i < ly.b; ++i)
            h[i] = static_cast<float>(nd(rng));
    }
    std::normal_distribution<double> nh(0.0, std::sqrt(1.0 / d->ch[0]));
    for (int i = 0; i < d->ch[0]; ++i)
        h[d->head + i] = static_cast<float>(nh(rng));
    NN_CUDA(nn::conv3Configure());
    NN_CUDA(nn::conv3TcConfigure());
    NN_CUDA(d->p.reserve(d->nParams));
    NN_CUDA(d->g.reserve(d->nParams));
    NN_CUDA(d->m.reserve(d->nParams));
    NN_CUDA(d->v.reserve(d->nParams));
    NN_CUDA(d->pb.reserve(d->nParams));
    NN_CUDA(d->wt.reserve(d->nWt));
    *out = d.release();
    const int rc = dxmcg_denoiser_set_params(*out, h.data());
    if (rc != DXMCG_OK) {
        delete *out;
        *out = nullptr;
    }
    return rc;
}

DXMCG_API void dxmcg_denoiser_destroy(dxmcg_denoiser* d)
{
    if (!d)
        return;
    cudaSetDevice(d->device);
    cudaDeviceSynchronize();
    delete d;
}

DXMCG_API int dxmcg_denoiser_set_wait_limit(dxmcg_denoiser* d, uint32_t polls)
{
    if (!d)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_set_wait_limit: null denoiser");
    d->waitPolls = polls;
    return DXMCG_OK;
}

DXMCG_API int dxmcg_denoiser_param_count(const dxmcg_denoiser* d, uint64_t* n)
{
    if (!d || !n)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_param_count: null argument");
    *n = d->nParams;
    return DXMCG_OK;
}

DXMCG_API int dxmcg_denoiser_get_params(dxmcg_denoiser* d, float* host)
{
    int rc = checkNet(d);
    if (rc != DXMCG_OK)
        return rc;
    if (!host)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_get_params: null output");
    NN_CUDA(cudaDeviceSynchronize());
    NN_CUDA(cudaMemcpy(host, d->p.p, d->nParams * sizeof(float), cudaMemcpyDeviceToHost));
    return DXMCG_OK;
}

DXMCG_API int dxmcg_denoiser_set_params(dxmcg_denoiser* d, const float* host)
{
    int rc = checkNet(d);
    if (rc != DXMCG_OK)
        return rc;
    if (!host)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_set_params: null input");
    NN_CUDA(cudaDeviceSynchronize());
    NN_CUDA(cudaMemcpy(d->p.p, host, d->nParams * sizeof(float), cudaMemcpyHostToDevice));
    NN_CUDA(cudaMemset(d->m.p, 0, d->nParams * sizeof(float)));
    NN_CUDA(cudaMemset(d->v.p, 0, d->nParams * sizeof(float)));
    NN_CUDA(cudaMemset(d->g.p, 0, d->nParams * sizeof(float)));
    d->step = 0;
    NN_CUDA(nn::launchToBf16(d->p.p, d->pb.p, d->nParams, nullptr));
    if ((rc = refreshWeights(d, nullptr)) != DXMCG_OK)
        return rc;
    NN_CUDA(cudaDeviceSynchronize());
    return DXMCG_OK;
}

DXMCG_API int dxmcg_denoiser_get_grads(dxmcg_denoiser* d, float* host)
{
    int rc = checkNet(d);
    if (rc != DXMCG_OK)
        return rc;
    if (!host)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_get_grads: null output");
    NN_CUDA(cudaDeviceSynchronize());
    NN_CUDA(cudaMemcpy(host, d->g.p, d->nParams * sizeof(float), cudaMemcpyDeviceToHost));
    return DXMCG_OK;
}

DXMCG_API int dxmcg_denoiser_forward(dxmcg_denoiser* d, const void* input, int B, int D, int H, int W, float* pred,
    void* cuda_stream)
{
    int rc = checkNet(d);
    if (rc != DXMCG_OK)
        return rc;
    if (!input || !pred)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_forward: null array");
    if ((rc = ensureShape(d, B, D, H, W)) != DXMCG_OK)
        return rc;
    const auto s = static_cast<cudaStream_t>(cuda_stream);
    if ((rc = forward(d, static_cast<const bf16*>(input), s, pred)) != DXMCG_OK)
        return rc;
    return DXMCG_OK;
}

DXMCG_API int dxmcg_denoiser_backward(dxmcg_denoiser* d, const void* input, const float* target, int B, int D,
    int H, int W, double* loss, void* cuda_stream)
{
    int rc = checkNet(d);
    if (rc != DXMCG_OK)
        return rc;
    if (!input || !target)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_backward: null array");
    if ((rc = ensureShape(d, B, D, H, W)) != DXMCG_OK)
        return rc;
    const auto s = static_cast<cudaStream_t>(cuda_stream);
    const auto* in = static_cast<const bf16*>(input);
    if ((rc = forward(d, in, s)) != DXMCG_OK)
        return rc;
    if ((rc = backward(d, in, target, s)) != DXMCG_OK)
        return rc;
    if (loss) {
        double h = 0;
        NN_CUDA(cudaMemcpyAsync(&h, d->loss.p, sizeof(double), cudaMemcpyDeviceToHost, s));
        NN_CUDA(cudaStreamSynchronize(s));
        *loss = h / static_cast<double>(d->nvox(0));
        if ((rc = tensorCoreStatus(d)) != DXMCG_OK)
            return rc;
    }
    return DXMCG_OK;
}

DXMCG_API int dxmcg_denoiser_adam(dxmcg_denoiser* d, float lr, void* cuda_stream)
{
    int rc = checkNet(d);
    if (rc != DXMCG_OK)
        return rc;
    const auto s = static_cast<cudaStream_t>(cuda_stream);
    const double b1 = 0.9, b2 = 0.999;
    ++d->step;
    const float c1 = static_cast<float>(1.0 / (1.0 - std::pow(b1, static_cast<double>(d->step))));
    const float c2 = static_cast<float>(1.0 / (1.0 - std::pow(b2, static_cast<double>(d->step))));
    NN_CUDA(nn::launchAdam(d->p.p, d->g.p, d->m.p, d->v.p, d->pb.p, d->nParams, lr, static_cast<float>(b1),
        static_cast<float>(b2), 1e-8f, c1, c2, s));
    return refreshWeights(d, s);
}

DXMCG_API int dxmcg_denoiser_prepare_input(const float* dose, const float* density, const uint8_t* material,
    uint64_t n, double scale, void* input, void* cuda_stream)
{
    if (n == 0)
        return DXMCG_OK;
    if (!dose || !density || !material || !input || !(scale > 0.0))
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_prepare_input: null array or scale <= 0");
    NN_CUDA(nn::launchPrepareInput(dose, density, material, nullptr, nullptr, 0.0, n, static_cast<float>(1.0 / scale),
        static_cast<bf16*>(input), static_cast<cudaStream_t>(cuda_stream)));
    return DXMCG_OK;
}

DXMCG_API int dxmcg_denoiser_gather_patches(const void* const* inputs, const float* const* targets,
    const int32_t* dims, int n_volumes, const int32_t* origins, int n_patch, int P, void* input_batch,
    float* target_batch, void* cuda_stream)
{
    if (n_volumes < 1 || n_patch < 1 || P < 1 || !inputs || !targets || !dims || !origins || !input_batch
        || !target_batch)
        return fail(DXMCG_ERR_ARGUMENT, "denoiser_gather_patches: bad arguments");
    NN_CUDA(nn::launchGatherPatches(reinterpret_cast<const bf16* const*>(inputs), targets, dims, n_volumes, origins,
        n_patch, P, static_cast<bf16*>(input_batch), target_batch, static_cast<cudaStream_t>(cuda_stream)));
    return DXMCG_OK;
}

} // extern "C"
