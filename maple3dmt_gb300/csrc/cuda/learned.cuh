// Learned preconditioner network: a 3-D convolutional network on a dense
// grid, trained and run with BF16 tcgen05 tensor-core kernels (FP32
// accumulation in tensor memory).  No counterpart in the reference, whose
// solve is SSOR-BiCGStab only; the network enters the solve as an extra
// direction of a flexible Krylov method (solver.cu), never as the judge of
// convergence.
//
// Data layout: activations are [n][D][H][W][32] BF16 (channels last, every
// layer padded to 32 channels), weights [27 taps][32 c_out][32 c_in] BF16
// with tap t = (dz + 1) 9 + (dy + 1) 3 + (dx + 1); the FP32 master copies and
// Adam moments live beside them.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

namespace m3d {
namespace learn {

constexpr int kCh = 32;        // channels of every activation tensor
constexpr int kTaps = 27;
constexpr int kWElems = kTaps * kCh * kCh;

class Cnn {
public:
    // layers >= 2, 1 <= c_in, c_out <= 32, hidden <= 32; weights He-initialised
    // from `seed` (first and hidden layers), biases zero.
    Cnn(int device, int layers, int c_in, int hidden, int c_out, unsigned seed);
    ~Cnn();
    Cnn(const Cnn&) = delete;
    Cnn& operator=(const Cnn&) = delete;

    int layers() const { return L; }
    int c_in() const { return cin; }
    int c_out() const { return cout; }
    // host FP32 copies: w [L][27][32][32] (padded), b [L][32]
    void get_weights(float* w, float* b) const;
    void set_weights(const float* w, const float* b);

    // Buffers for n samples of a D x H x W grid (W in {16, 32, 64, 128}, H a
    // multiple of 128 / W).
    void ensure(int n, int D, int H, int W);
    // input activations: [n][D][H][W][32] BF16, channels >= c_in zero
    __nv_bfloat16* input() { return act[0]; }
    // the network on the first n samples of input(); output FP32 [n V][c_out]
    const float* forward(int n);
    // gradients of sum(dout * out) for dout FP32 [n V][c_out] (after forward(n));
    // into the FP32 gradient buffers; d/dinput to dx ([n V][32] FP32) if given
    void backward(int n, const float* dout, float* dx);
    // 0.5 * mean over samples and voxels of |out - target|^2 and its backward
    double loss_backward(int n, const float* target);
    void adam_step(float lr, float beta1 = 0.9f, float beta2 = 0.999f, float eps = 1e-8f);
    // host FP32 gradients: dw [L][27][32][32], db [L][32]
    void get_grads(float* dw, float* db) const;
    unsigned error_flag();
    cudaStream_t stream() const { return st; }
    // run on the caller's stream (the caller keeps ownership; null: the
    // network's own stream again)
    void set_stream(cudaStream_t s) { st = s ? s : own_st; }

private:
    int dev, L, cin, hid, cout;
    int n_cap = 0, D = 0, H = 0, W = 0, V = 0;
    int bw = 0, bh = 0;
    cudaStream_t st = nullptr;       // the stream launches go to
    cudaStream_t own_st = nullptr;   // created and destroyed by this object
    std::vector<int> ci, co;                 // channels in / out of each layer
    float *w32 = nullptr, *b32 = nullptr;    // FP32 masters
    float *mw = nullptr, *vw = nullptr, *mb = nullptr, *vb = nullptr;
    float *gw = nullptr, *gb = nullptr;      // gradients
    __nv_bfloat16 *wbf = nullptr, *wtbf = nullptr;   // forward and transposed (dgrad) weights
    std::vector<__nv_bfloat16*> act;        // L + 1 activation buffers
    __nv_bfloat16* delta[2] = {nullptr, nullptr};
    float* out32 = nullptr;
    float* dout32 = nullptr;
    __nv_bfloat16 *xcol = nullptr, *dyt = nullptr;
    float* ws = nullptr;
    double* red = nullptr;
    unsigned* err = nullptr;
    int* dch = nullptr;                      // device copy of ci, co
    int splits = 0;
    long long adam_t = 0;
    std::vector<CUtensorMap> act_map, delta_map, w_map, wt_map;
    // the same buffers with a halo box (W <= 64): a tile's input and its
    // one-voxel border in y and z, loaded once per x shift
    std::vector<CUtensorMap> act_hmap, delta_hmap;
    CUtensorMap xcol_map{}, dyt_map{};
    void free_grid();
    void upload_bf16();
    void conv(int l, bool transposed, const CUtensorMap& in_map, const CUtensorMap& in_hmap,
              const __nv_bfloat16* mask, __nv_bfloat16* out, float* o32, int n32, int n);
    void wgrad(int l, const __nv_bfloat16* x, const __nv_bfloat16* d, int n);
};

// ---------------------------------------------------------------------------
// Dense-grid view of an edge field (the network's input and output)
// ---------------------------------------------------------------------------

// Per mesh: the dense grid of G^3 cells (G = 2^level of the octree's unit
// cube), the edge rows of every (cell, direction) and the cell of every row,
// and the leaves of every cell (for the conductivity channel).
struct GridMap {
    int G = 0, n_cells = 0;        // n_cells = G^3
    int n_pad = 0;
    int* cd_ptr = nullptr;         // [3 n_cells + 1] rows of (cell, direction) key 3 c + d
    int* cd_row = nullptr;         // permuted rows
    int* row_cell = nullptr;       // [n_pad] dense cell of a free row, -1 otherwise
    signed char* row_dir = nullptr;  // [n_pad]
    int* sig_ptr = nullptr;        // [n_cells + 1] leaves of a cell
    int* sig_leaf = nullptr;
    float* sig_feat = nullptr;     // [n_cells] conductivity channel of the current model
};

constexpr int kInCh = 8;           // residual (Re, Im) x 3 directions, conductivity, frequency
constexpr int kOutCh = 6;          // error (Re, Im) x 3 directions

// conductivity channel (log10 sigma + 2) / 3 averaged over a cell's leaves
void grid_sigma_feature(const GridMap& g, const double* sigma, cudaStream_t s);
// network input of K lanes of an edge vector ([n_pad][K], FP64 or FP32
// complex): per (cell, direction) means of the lane's values, scaled by the
// lane's RMS over the grid, the conductivity channel and the frequency
// channel log10(f) / 3; BF16 [K][G^3][32].  work: FP32 [K][G^3][6] + K.
void grid_features(const GridMap& g, const double2* v, int K, const double* freq_of_lane, __nv_bfloat16* in,
                   float* work, cudaStream_t s);
void grid_features(const GridMap& g, const float2* v, int K, const double* freq_of_lane, __nv_bfloat16* in,
                   float* work, cudaStream_t s);
// the same means as FP32 [K][G^3][6], unscaled (training targets)
void grid_means(const GridMap& g, const double2* v, int K, float* out, cudaStream_t s);
// z[row][k] = out[k][cell(row)][2 dir + (0, 1)] (zero on rows without a cell)
void grid_prolong(const GridMap& g, const float* out, int K, float2* z, cudaStream_t s);

// Tensor maps (driver entry point reached through the runtime, no -lcuda).
void encode_act_map(CUtensorMap* m, const void* base, int n, int D, int H, int W, int bw, int bh, int halo = 0);
void encode_2d_map(CUtensorMap* m, const void* base, long long cols, int rows, int box_rows);

}  // namespace learn
}  // namespace m3d
