// Device kernels of the learned-guess MLP (16 -> 64 -> 64 -> 4, tanh, FP32):
// tiled forward pass, back-propagation into per-block partial gradients,
// and a fused gradient-sum + Adam update (Kingma & Ba 2015, Algorithm 1,
// with bias correction).  A block takes a tile of 128 samples; weights,
// the input tile and both hidden activations stay in shared memory, so a
// sample's data is read from HBM once and the hidden layers never leave the
// SM.  Partial gradients are summed in a fixed block order, so results are
// deterministic.
#include "fe_mlp.h"

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/feng_cuda.h"
#include "fe_common.h"

namespace feng {

#define CKM(x)                                                                         \
  do {                                                                                 \
    cudaError_t _e = (x);                                                              \
    if(_e != cudaSuccess) {                                                            \
      set_error("CUDA error %s at %s:%d", cudaGetErrorString(_e), __FILE__, __LINE__); \
      return FE_CUDA_FAIL;                                                             \
    }                                                                                  \
  } while(0)

namespace {

using D = MLPDims;
constexpr int THREADS = 256;
constexpr int LDX = D::NIN + 1;  // padded leading dimensions (bank spread)
constexpr int LDA = D::H + 1;
constexpr int LDW3 = D::H + 1;

// Shared-memory layout (floats); every offset is a multiple of 4.
constexpr int S_W1T = 0;                         // [NIN x H]  W1 transposed
constexpr int S_B1 = S_W1T + D::NIN * D::H;      // [H]
constexpr int S_W2T = S_B1 + D::H;               // [H x H]    W2 transposed
constexpr int S_W2 = S_W2T + D::H * D::H;        // [H x H]    W2 (backward only)
constexpr int S_B2 = S_W2 + D::H * D::H;         // [H]
constexpr int S_W3 = S_B2 + D::H;                // [NOUT x LDW3]
constexpr int S_B3 = S_W3 + D::NOUT * LDW3;      // [NOUT]
constexpr int S_X = S_B3 + D::NOUT;              // [TILE x LDX]
constexpr int S_A1 = S_X + D::TILE * LDX;        // [TILE x LDA]
constexpr int S_A2 = S_A1 + D::TILE * LDA;       // [TILE x LDA]
constexpr int S_Y = S_A2 + D::TILE * LDA;        // [TILE x NOUT]
constexpr int S_END = S_Y + D::TILE * D::NOUT;
static_assert(S_B1 % 4 == 0 && S_W2T % 4 == 0 && S_W2 % 4 == 0 && S_X % 4 == 0 && S_A1 % 4 == 0 &&
                  S_A2 % 4 == 0 && S_Y % 4 == 0,
              "shared offsets must keep float4 alignment");
constexpr size_t SMEM_BYTES = sizeof(float) * S_END;

static_assert(D::TILE == 128 && THREADS == 256 && D::H == 64, "thread mapping assumes these sizes");

// C[TILE x 64] (ldc) from A[TILE x K] (lda) and Bt[K x 64]:
//   MODE 0: C = tanh(A Bt + bias)
//   MODE 1: C = (A Bt) * (1 - C^2)   (tanh derivative, C holds the activations)
// Thread (tx = t % 16, ty = t / 16) owns rows 8 ty .. 8 ty + 7, columns 4 tx .. 4 tx + 3.
template <int K, int MODE>
__device__ __forceinline__ void dense64(const float *A, int lda, const float *Bt, const float *bias, float *C,
                                        int ldc)
{
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[8][4];
#pragma unroll
  for(int r = 0; r < 8; ++r)
#pragma unroll
    for(int c = 0; c < 4; ++c) acc[r][c] = MODE == 0 ? bias[tx * 4 + c] : 0.f;
#pragma unroll 4
  for(int k = 0; k < K; ++k) {
    const float4 b = *reinterpret_cast<const float4 *>(Bt + k * 64 + tx * 4);
#pragma unroll
    for(int r = 0; r < 8; ++r) {
      const float a = A[(ty * 8 + r) * lda + k];
      acc[r][0] = fmaf(a, b.x, acc[r][0]);
      acc[r][1] = fmaf(a, b.y, acc[r][1]);
      acc[r][2] = fmaf(a, b.z, acc[r][2]);
      acc[r][3] = fmaf(a, b.w, acc[r][3]);
    }
  }
#pragma unroll
  for(int r = 0; r < 8; ++r)
#pragma unroll
    for(int c = 0; c < 4; ++c) {
      float *p = C + (ty * 8 + r) * ldc + tx * 4 + c;
      if(MODE == 0)
        *p = tanhf(acc[r][c]);
      else {
        const float h = *p;
        *p = acc[r][c] * (1.f - h * h);
      }
    }
}

__device__ __forceinline__ void load_weights(const float *__restrict__ w, float *sm, bool withW2)
{
  for(int e = threadIdx.x; e < D::H * D::NIN; e += THREADS) {
    const int j = e / D::NIN, k = e % D::NIN;
    sm[S_W1T + k * D::H + j] = w[D::OW1 + e];
  }
  for(int e = threadIdx.x; e < D::H * D::H; e += THREADS) {
    const int j = e / D::H, k = e % D::H;
    const float v = w[D::OW2 + e];
    sm[S_W2T + k * D::H + j] = v;
    if(withW2) sm[S_W2 + e] = v;
  }
  for(int e = threadIdx.x; e < D::NOUT * D::H; e += THREADS) {
    const int o = e / D::H, k = e % D::H;
    sm[S_W3 + o * LDW3 + k] = w[D::OW3 + e];
  }
  if(threadIdx.x < D::H) {
    sm[S_B1 + threadIdx.x] = w[D::OB1 + threadIdx.x];
    sm[S_B2 + threadIdx.x] = w[D::OB2 + threadIdx.x];
  }
  if(threadIdx.x < D::NOUT) sm[S_B3 + threadIdx.x] = w[D::OB3 + threadIdx.x];
}

// Row of sample r of this tile (-1: past the end).
__device__ __forceinline__ int64_t tile_row(int64_t base, int r, int64_t n, const int32_t *idx)
{
  const int64_t i = base + r;
  if(i >= n) return -1;
  return idx ? (int64_t)idx[i] : i;
}

// Input tile, both hidden layers and the outputs (in S_Y) of one tile.
__device__ __forceinline__ void tile_forward(const float *__restrict__ X, int64_t n, const int32_t *idx,
                                             float *sm)
{
  const int64_t base = (int64_t)blockIdx.x * D::TILE;
  for(int e = threadIdx.x; e < D::TILE * D::NIN; e += THREADS) {
    const int r = e / D::NIN, k = e % D::NIN;
    const int64_t row = tile_row(base, r, n, idx);
    sm[S_X + r * LDX + k] = row >= 0 ? X[row * D::NIN + k] : 0.f;
  }
  __syncthreads();
  dense64<D::NIN, 0>(sm + S_X, LDX, sm + S_W1T, sm + S_B1, sm + S_A1, LDA);
  __syncthreads();
  dense64<D::H, 0>(sm + S_A1, LDA, sm + S_W2T, sm + S_B2, sm + S_A2, LDA);
  __syncthreads();
  for(int e = threadIdx.x; e < D::TILE * D::NOUT; e += THREADS) {
    const int r = e / D::NOUT, o = e % D::NOUT;
    float y = sm[S_B3 + o];
    const float *a = sm + S_A2 + r * LDA, *w = sm + S_W3 + o * LDW3;
#pragma unroll 8
    for(int k = 0; k < D::H; ++k) y = fmaf(a[k], w[k], y);
    sm[S_Y + e] = y;
  }
  __syncthreads();
}

__global__ void __launch_bounds__(THREADS) k_mlp_forward(const float *__restrict__ w, const float *__restrict__ X,
                                                         int64_t n, float *__restrict__ Y)
{
  extern __shared__ __align__(16) float sm[];
  load_weights(w, sm, false);
  tile_forward(X, n, nullptr, sm);
  const int64_t base = (int64_t)blockIdx.x * D::TILE;
  for(int e = threadIdx.x; e < D::TILE * D::NOUT; e += THREADS) {
    const int64_t i = base + e / D::NOUT;
    if(i < n) Y[i * D::NOUT + e % D::NOUT] = sm[S_Y + e];
  }
}

// Back-propagation of one tile into partial[blockIdx.x * P + ...].
__global__ void __launch_bounds__(THREADS) k_mlp_grad(const float *__restrict__ w, const float *__restrict__ X,
                                                      const float *__restrict__ T, const float *__restrict__ M,
                                                      const int32_t *__restrict__ idx, int64_t nb, float scale,
                                                      float *__restrict__ partial, float *__restrict__ lossPart)
{
  extern __shared__ __align__(16) float sm[];
  __shared__ float red[THREADS / 32];
  load_weights(w, sm, true);
  tile_forward(X, nb, idx, sm);
  const int64_t base = (int64_t)blockIdx.x * D::TILE;
  float *g = partial + (int64_t)blockIdx.x * D::P;

  // dL/dy = 2 scale mask (y - t)
  float loss = 0.f;
  for(int e = threadIdx.x; e < D::TILE * D::NOUT; e += THREADS) {
    const int r = e / D::NOUT, o = e % D::NOUT;
    const int64_t row = tile_row(base, r, nb, idx);
    float d = 0.f;
    if(row >= 0) {
      const float m = M[row * D::NOUT + o];
      const float err = sm[S_Y + e] - T[row * D::NOUT + o];
      loss += m * err * err * scale;
      d = 2.f * m * err * scale;
    }
    sm[S_Y + e] = d;
  }
  for(int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
  if((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = loss;
  __syncthreads();
  if(threadIdx.x == 0) {
    float s = 0.f;
    for(int k = 0; k < THREADS / 32; ++k) s += red[k];
    lossPart[blockIdx.x] = s;
  }

  // Output layer: gW3[o][k] = sum_r dY[r][o] A2[r][k], gb3[o] = sum_r dY[r][o].
  {
    const int o = threadIdx.x / D::H, k = threadIdx.x % D::H;  // 256 = 4 x 64 entries
    float acc = 0.f;
    for(int r = 0; r < D::TILE; ++r) acc = fmaf(sm[S_Y + r * D::NOUT + o], sm[S_A2 + r * LDA + k], acc);
    g[D::OW3 + o * D::H + k] = acc;
    if(threadIdx.x < D::NOUT) {
      float b = 0.f;
      for(int r = 0; r < D::TILE; ++r) b += sm[S_Y + r * D::NOUT + threadIdx.x];
      g[D::OB3 + threadIdx.x] = b;
    }
  }
  __syncthreads();
  // D2 = (dY W3) * (1 - A2^2), in place of A2.
  for(int e = threadIdx.x; e < D::TILE * D::H; e += THREADS) {
    const int r = e / D::H, k = e % D::H;
    float s = 0.f;
#pragma unroll
    for(int o = 0; o < D::NOUT; ++o) s = fmaf(sm[S_Y + r * D::NOUT + o], sm[S_W3 + o * LDW3 + k], s);
    float *p = sm + S_A2 + r * LDA + k;
    const float h = *p;
    *p = s * (1.f - h * h);
  }
  __syncthreads();
  // gW2[j][k] = sum_r D2[r][j] A1[r][k], gb2[j] = sum_r D2[r][j]: thread owns j = t/4, 16 k's.
  {
    const int j = threadIdx.x >> 2, kq = (threadIdx.x & 3) * 16;
    float acc[16], accb = 0.f;
#pragma unroll
    for(int c = 0; c < 16; ++c) acc[c] = 0.f;
    for(int r = 0; r < D::TILE; ++r) {
      const float d = sm[S_A2 + r * LDA + j];
      accb += d;
#pragma unroll
      for(int c = 0; c < 16; ++c) acc[c] = fmaf(d, sm[S_A1 + r * LDA + kq + c], acc[c]);
    }
#pragma unroll
    for(int c = 0; c < 16; ++c) g[D::OW2 + j * D::H + kq + c] = acc[c];
    if((threadIdx.x & 3) == 0) g[D::OB2 + j] = accb;
  }
  __syncthreads();
  // D1 = (D2 W2) * (1 - A1^2), in place of A1.
  dense64<D::H, 1>(sm + S_A2, LDA, sm + S_W2, nullptr, sm + S_A1, LDA);
  __syncthreads();
  // gW1[j][k] = sum_r D1[r][j] X[r][k], gb1[j] = sum_r D1[r][j]: thread owns j = t/4, 4 k's.
  {
    const int j = threadIdx.x >> 2, kq = (threadIdx.x & 3) * 4;
    float acc[4] = {0.f, 0.f, 0.f, 0.f}, accb = 0.f;
    for(int r = 0; r < D::TILE; ++r) {
      const float d = sm[S_A1 + r * LDA + j];
      accb += d;
#pragma unroll
      for(int c = 0; c < 4; ++c) acc[c] = fmaf(d, sm[S_X + r * LDX + kq + c], acc[c]);
    }
#pragma unroll
    for(int c = 0; c < 4; ++c) g[D::OW1 + j * D::NIN + kq + c] = acc[c];
    if((threadIdx.x & 3) == 0) g[D::OB1 + j] = accb;
  }
}

// Gradient = sum of the block partials (fixed order), then Adam.
__global__ void __launch_bounds__(256) k_mlp_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                                                  const float *__restrict__ partial, int nblocks, float lr,
                                                  float beta1, float beta2, float eps, float c1, float c2,
                                                  float *__restrict__ gradOut, const float *__restrict__ lossPart,
                                                  float *__restrict__ lossOut)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if(p < D::P) {
    float gsum = 0.f;
    for(int b = 0; b < nblocks; ++b) gsum += partial[(int64_t)b * D::P + p];
    if(gradOut) gradOut[p] = gsum;
    const float mi = beta1 * m[p] + (1.f - beta1) * gsum;
    const float vi = beta2 * v[p] + (1.f - beta2) * gsum * gsum;
    m[p] = mi;
    v[p] = vi;
    w[p] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
  if(lossOut && blockIdx.x == 0 && threadIdx.x == 0) {
    float s = 0.f;
    for(int b = 0; b < nblocks; ++b) s += lossPart[b];
    *lossOut = s;
  }
}

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

__global__ void k_mlp_sample(uint64_t key, int64_t nRows, int64_t nb, int32_t *__restrict__ idx)
{
  for(int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x)
    idx[i] = (int32_t)(mix64(key + 0x9e3779b97f4a7c15ULL * (uint64_t)(i + 1)) % (uint64_t)nRows);
}

double splitmix_uniform(uint64_t &state)
{
  uint64_t z = (state += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

}  // namespace

MLPDevice::~MLPDevice()
{
  cudaFree(params_);
  cudaFree(m_);
  cudaFree(v_);
  cudaFree(partial_);
  cudaFree(lossPart_);
}

int MLPDevice::init(uint64_t seed, int64_t maxBatch, cudaStream_t s, float outScale)
{
  if(maxBatch < 1) {
    set_error("MLP batch capacity must be positive");
    return FE_INVALID_ARG;
  }
  s_ = s;
  seed_ = seed;
  maxBatch_ = maxBatch;
  maxBlocks_ = (int)((maxBatch + D::TILE - 1) / D::TILE);
  std::vector<float> w(D::P, 0.f);
  uint64_t st = seed;
  auto fill = [&](int off, int fanOut, int fanIn, float extra) {
    const double a = std::sqrt(6.0 / (fanIn + fanOut));
    for(int e = 0; e < fanOut * fanIn; ++e) w[off + e] = (float)(extra * a * (2.0 * splitmix_uniform(st) - 1.0));
  };
  fill(D::OW1, D::H, D::NIN, 1.f);
  fill(D::OW2, D::H, D::H, 1.f);
  fill(D::OW3, D::NOUT, D::H, outScale);
  CKM(cudaMalloc(&params_, sizeof(float) * D::P));
  CKM(cudaMalloc(&m_, sizeof(float) * D::P));
  CKM(cudaMalloc(&v_, sizeof(float) * D::P));
  CKM(cudaMalloc(&partial_, sizeof(float) * D::P * (size_t)maxBlocks_));
  CKM(cudaMalloc(&lossPart_, sizeof(float) * (size_t)maxBlocks_));
  CKM(cudaMemsetAsync(m_, 0, sizeof(float) * D::P, s_));
  CKM(cudaMemsetAsync(v_, 0, sizeof(float) * D::P, s_));
  CKM(cudaMemcpyAsync(params_, w.data(), sizeof(float) * D::P, cudaMemcpyHostToDevice, s_));
  CKM(cudaStreamSynchronize(s_));
  CKM(cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
  CKM(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES));
  step_ = 0;
  return FE_OK;
}

int MLPDevice::setParams(const float *hostParams)
{
  CKM(cudaMemcpyAsync(params_, hostParams, sizeof(float) * D::P, cudaMemcpyHostToDevice, s_));
  CKM(cudaMemsetAsync(m_, 0, sizeof(float) * D::P, s_));
  CKM(cudaMemsetAsync(v_, 0, sizeof(float) * D::P, s_));
  CKM(cudaStreamSynchronize(s_));
  step_ = 0;
  return FE_OK;
}

int MLPDevice::getParams(float *hostParams) const
{
  CKM(cudaMemcpyAsync(hostParams, params_, sizeof(float) * D::P, cudaMemcpyDeviceToHost, s_));
  CKM(cudaStreamSynchronize(s_));
  return FE_OK;
}

int MLPDevice::forward(const float *X, int64_t n, float *Y)
{
  if(n <= 0) return FE_OK;
  const int64_t blocks = (n + D::TILE - 1) / D::TILE;
  (k_mlp_forward<<<(unsigned)blocks, THREADS, SMEM_BYTES, s_>>>(params_, X, n, Y), ::feng::count_launch());
  CKM(cudaGetLastError());
  return FE_OK;
}

int MLPDevice::gradient(const float *X, const float *T, const float *M, const int32_t *idx, int64_t nb)
{
  if(nb <= 0 || nb > maxBatch_) {
    set_error("MLP batch of %lld samples outside 1..%lld", (long long)nb, (long long)maxBatch_);
    return FE_INVALID_ARG;
  }
  lastBlocks_ = (int)((nb + D::TILE - 1) / D::TILE);
  const float scale = (float)(1.0 / ((double)nb * D::NOUT));
  (k_mlp_grad<<<lastBlocks_, THREADS, SMEM_BYTES, s_>>>(params_, X, T, M, idx, nb, scale, partial_, lossPart_),
   ::feng::count_launch());
  CKM(cudaGetLastError());
  return FE_OK;
}

int MLPDevice::adam(float lr, float beta1, float beta2, float eps, float *gradOut, float *lossOut)
{
  if(lastBlocks_ < 1) {
    set_error("MLP Adam step without a gradient");
    return FE_INVALID_ARG;
  }
  ++step_;
  const float c1 = (float)(1.0 - std::pow((double)beta1, step_));
  const float c2 = (float)(1.0 - std::pow((double)beta2, step_));
  (k_mlp_adam<<<(D::P + 255) / 256, 256, 0, s_>>>(params_, m_, v_, partial_, lastBlocks_, lr, beta1, beta2, eps,
                                                   c1, c2, gradOut, lossPart_, lossOut),
   ::feng::count_launch());
  CKM(cudaGetLastError());
  return FE_OK;
}

int MLPDevice::sample(int64_t nRows, int64_t nb, int32_t *idx)
{
  if(nRows < 1 || nb < 1) return FE_INVALID_ARG;
  const uint64_t key = seed_ * 0xd1b54a32d192ed03ULL + (++draws_);
  const int blocks = (int)std::min<int64_t>((nb + 255) / 256, 4096);
  (k_mlp_sample<<<blocks, 256, 0, s_>>>(key, nRows, nb, idx), ::feng::count_launch());
  CKM(cudaGetLastError());
  return FE_OK;
}

}  // namespace feng

// ---- C ABI: host-buffer entry points around the same kernels -------------------

using namespace feng;

struct fe_mlp {
  MLPDevice net;
  cudaStream_t s = nullptr;
  float *x = nullptr, *t = nullptr, *m = nullptr, *y = nullptr, *g = nullptr, *loss = nullptr;
  int64_t cap = 0;
  ~fe_mlp()
  {
    cudaFree(x);
    cudaFree(t);
    cudaFree(m);
    cudaFree(y);
    cudaFree(g);
    cudaFree(loss);
    if(s) cudaStreamDestroy(s);
  }
  int reserve(int64_t n)
  {
    if(n <= cap) return FE_OK;
    cudaFree(x);
    cudaFree(t);
    cudaFree(m);
    cudaFree(y);
    x = t = m = y = nullptr;
    CKM(cudaMalloc(&x, sizeof(float) * n * D::NIN));
    CKM(cudaMalloc(&t, sizeof(float) * n * D::NOUT));
    CKM(cudaMalloc(&m, sizeof(float) * n * D::NOUT));
    CKM(cudaMalloc(&y, sizeof(float) * n * D::NOUT));
    cap = n;
    return FE_OK;
  }
};

extern "C" {

int fe_mlp_sizes(int *nin, int *h1, int *h2, int *nout, int64_t *nparams)
{
  if(nin) *nin = D::NIN;
  if(h1) *h1 = D::H;
  if(h2) *h2 = D::H;
  if(nout) *nout = D::NOUT;
  if(nparams) *nparams = D::P;
  return FE_OK;
}

int fe_mlp_create(uint64_t seed, int64_t max_batch, fe_mlp **out)
{
  if(!out || max_batch < 1) {
    set_error("fe_mlp_create: null output or non-positive batch capacity");
    return FE_INVALID_ARG;
  }
  fe_mlp *h = new fe_mlp();
  cudaError_t e = cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking);
  int st = e == cudaSuccess ? FE_OK : FE_CUDA_FAIL;
  if(e != cudaSuccess) set_error("fe_mlp_create: %s", cudaGetErrorString(e));
  if(st == FE_OK) st = h->net.init(seed, max_batch, h->s);
  if(st == FE_OK && cudaMalloc(&h->g, sizeof(float) * D::P) != cudaSuccess) st = FE_CUDA_FAIL;
  if(st == FE_OK && cudaMalloc(&h->loss, sizeof(float)) != cudaSuccess) st = FE_CUDA_FAIL;
  if(st != FE_OK) {
    delete h;
    return st;
  }
  *out = h;
  return FE_OK;
}

void fe_mlp_destroy(fe_mlp *h) { delete h; }

int fe_mlp_set_params(fe_mlp *h, const float *params)
{
  if(!h || !params) return FE_INVALID_ARG;
  return h->net.setParams(params);
}

int fe_mlp_get_params(fe_mlp *h, float *params)
{
  if(!h || !params) return FE_INVALID_ARG;
  return h->net.getParams(params);
}

int fe_mlp_forward(fe_mlp *h, const float *x, int64_t n, float *y)
{
  if(!h || !x || !y || n < 0) return FE_INVALID_ARG;
  FE_TRY(h->reserve(n));
  CKM(cudaMemcpyAsync(h->x, x, sizeof(float) * n * D::NIN, cudaMemcpyHostToDevice, h->s));
  FE_TRY(h->net.forward(h->x, n, h->y));
  CKM(cudaMemcpyAsync(y, h->y, sizeof(float) * n * D::NOUT, cudaMemcpyDeviceToHost, h->s));
  CKM(cudaStreamSynchronize(h->s));
  return FE_OK;
}

// Gradient of the masked loss over the batch (x, t, mask), then one Adam step
// with learning rate lr (lr = 0 leaves the parameters unchanged; the moment
// estimates still advance).  grad (P floats) and loss receive the gradient
// and loss before the step.
int fe_mlp_train_step(fe_mlp *h, const float *x, const float *t, const float *mask, int64_t n, double lr,
                      float *grad, double *loss)
{
  if(!h || !x || !t || !mask || n < 1) return FE_INVALID_ARG;
  FE_TRY(h->reserve(n));
  CKM(cudaMemcpyAsync(h->x, x, sizeof(float) * n * D::NIN, cudaMemcpyHostToDevice, h->s));
  CKM(cudaMemcpyAsync(h->t, t, sizeof(float) * n * D::NOUT, cudaMemcpyHostToDevice, h->s));
  CKM(cudaMemcpyAsync(h->m, mask, sizeof(float) * n * D::NOUT, cudaMemcpyHostToDevice, h->s));
  FE_TRY(h->net.gradient(h->x, h->t, h->m, nullptr, n));
  FE_TRY(h->net.adam((float)lr, 0.9f, 0.999f, 1e-8f, h->g, h->loss));
  if(grad) CKM(cudaMemcpyAsync(grad, h->g, sizeof(float) * D::P, cudaMemcpyDeviceToHost, h->s));
  float l = 0.f;
  CKM(cudaMemcpyAsync(&l, h->loss, sizeof(float), cudaMemcpyDeviceToHost, h->s));
  CKM(cudaStreamSynchronize(h->s));
  if(loss) *loss = l;
  return FE_OK;
}

}  // extern "C"
