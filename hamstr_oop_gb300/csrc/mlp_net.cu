// ##################################################################
//
// mlp_net.cu -- the warm-start network: 5 -> 256 -> 256 -> 256 -> 4,
// GELU, BF16 weights and activations, FP32 accumulation
//
// Forward and backward passes are chains of the tcgen05 GEMM
// (mlp_gemm.cu) with fused epilogues; the small kernels here gather
// minibatches, form the loss gradient, reduce split-K partial sums and
// bias gradients in a fixed order, and apply Adam to FP32 master weights,
// re-deriving the BF16 copies (and the transposes the backward pass
// reads).  Shapes are padded for the tensor cores: the 5 inputs to 64
// columns, the 4 outputs to 16 rows (64 for the K of the first backward
// product); the padding stays exactly zero through training.
// ##################################################################
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "mlp.h"

namespace hamstr {
void set_last_error(const std::string& m);
}

using namespace hamstr;
using bf16 = __nv_bfloat16;

namespace {

constexpr int W = 256;       // hidden width
constexpr int NIN = 5, NOUT = 4;
constexpr int KIN = 64;      // padded input width
constexpr int NOP = 16;      // padded output rows of W4
constexpr int KOP = 64;      // padded K of dZ4 * W4

// logical parameter layout (host API): W1[256][5] b1 W2[256][256] b2
// W3[256][256] b3 W4[4][256] b4
constexpr int kNParams = W * NIN + W + 2 * (W * W + W) + NOUT * W + NOUT;

__device__ __forceinline__ unsigned long long mix64(unsigned long long x)
{
   // splitmix64 finaliser (Steele, Lea & Flood, 2014)
   x += 0x9E3779B97F4A7C15ull;
   x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
   x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
   return x ^ (x >> 31);
}

// minibatch rows: sample i of step `step` (seeded), or rows 0..B-1 in
// order when seed == 0; X padded to 64 columns, its transpose, targets
__global__ void gather_kernel(const float* __restrict__ feat, const float* __restrict__ targ, long long n_all, int B,
                              int B_valid, unsigned long long seed, unsigned long long step, bf16* __restrict__ X,
                              bf16* __restrict__ Xt, float* __restrict__ T)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= B) return;
   long long src = -1;
   if (i < B_valid) src = seed ? (long long)(mix64(seed ^ mix64(step * 0x100000001ull + i)) % (unsigned long long)n_all) : i;
   for (int k = 0; k < KIN; k++) {
      const float v = (src >= 0 && k < NIN) ? feat[src * NIN + k] : 0.f;
      const bf16 b = __float2bfloat16_rn(v);
      X[(size_t)i * KIN + k] = b;
      Xt[(size_t)k * B + i] = b;
   }
   if (T)
      for (int k = 0; k < NOUT; k++) T[(size_t)i * NOUT + k] = (src >= 0 && targ) ? targ[src * NOUT + k] : 0.f;
}

// loss = sum over valid rows of (y - t)^2 / (B_valid * 4); dY = 2 (y - t) / (B_valid * 4)
// into dZ4 [B][64] (columns >= 4 zero) and dZ4t [16][B] (rows >= 4 zero);
// per-block partial loss and output-bias gradient
__global__ void loss_kernel(const float* __restrict__ Y, const float* __restrict__ T, int B, int B_valid,
                            bf16* __restrict__ dZ, bf16* __restrict__ dZt, double* __restrict__ part)
{
   __shared__ double s_l[256], s_g[4][256];
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   double l = 0.0, g[4] = {0.0, 0.0, 0.0, 0.0};
   const float scale = 2.f / (float)(B_valid * NOUT);
   if (i < B) {
      for (int k = 0; k < KOP; k++) dZ[(size_t)i * KOP + k] = __float2bfloat16_rn(0.f);
      for (int k = 0; k < NOP; k++) {
         float d = 0.f;
         if (k < NOUT && i < B_valid) {
            const float e = Y[(size_t)i * NOUT + k] - T[(size_t)i * NOUT + k];
            l += (double)e * e;
            d = scale * e;
            g[k] = d;
         }
         const bf16 b = __float2bfloat16_rn(d);
         if (k < NOUT) dZ[(size_t)i * KOP + k] = b;
         dZt[(size_t)k * B + i] = b;
      }
   }
   s_l[threadIdx.x] = l;
   for (int k = 0; k < 4; k++) s_g[k][threadIdx.x] = g[k];
   __syncthreads();
   for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
         s_l[threadIdx.x] += s_l[threadIdx.x + s];
         for (int k = 0; k < 4; k++) s_g[k][threadIdx.x] += s_g[k][threadIdx.x + s];
      }
      __syncthreads();
   }
   if (threadIdx.x == 0) {
      part[5 * blockIdx.x] = s_l[0] / (double)(B_valid * NOUT);
      for (int k = 0; k < 4; k++) part[5 * blockIdx.x + 1 + k] = s_g[k][0];
   }
}

// out[r] = sum_b M[r][b] (BF16 rows of the transposed dZ), fixed order
__global__ void rowsum_kernel(const bf16* __restrict__ Mt, int B, float* __restrict__ out)
{
   __shared__ float s[256];
   const int r = blockIdx.x;
   float a = 0.f;
   for (int b = threadIdx.x; b < B; b += blockDim.x) a += __bfloat162float(Mt[(size_t)r * B + b]);
   s[threadIdx.x] = a;
   __syncthreads();
   for (int k = blockDim.x / 2; k > 0; k >>= 1) {
      if (threadIdx.x < k) s[threadIdx.x] += s[threadIdx.x + k];
      __syncthreads();
   }
   if (threadIdx.x == 0) out[r] = s[0];
}

// out = sum over splits of part[s], in split order
__global__ void splitk_kernel(const float* __restrict__ part, int splits, int n, float* __restrict__ out)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) return;
   float a = 0.f;
   for (int s = 0; s < splits; s++) a += part[(size_t)s * n + i];
   out[i] = a;
}

// Adam (Kingma & Ba, 2015) on one FP32 tensor [rows][cols]; the gradient
// may be stored transposed ([cols][rows]).  Writes the BF16 copy
// [rows][ldw] and, when wt != nullptr, the transpose [cols][ldt].
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, int g_transposed, float* __restrict__ m,
                            float* __restrict__ v, int rows, int cols, float lr, float b1, float b2, float eps,
                            float c1, float c2, bf16* __restrict__ w, int ldw, bf16* __restrict__ wt, int ldt)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= rows * cols) return;
   const int r = i / cols, c = i - r * cols;
   const float gi = g_transposed ? g[(size_t)c * rows + r] : g[i];
   const float mi = b1 * m[i] + (1.f - b1) * gi;
   const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
   m[i] = mi;
   v[i] = vi;
   const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
   p[i] = pi;
   if (w) {
      const bf16 b = __float2bfloat16_rn(pi);
      w[(size_t)r * ldw + c] = b;
      if (wt) wt[(size_t)c * ldt + r] = b;
   }
}

// BF16 copies of an FP32 tensor [rows][cols] (no update)
__global__ void cast_kernel(const float* __restrict__ p, int rows, int cols, bf16* __restrict__ w, int ldw,
                            bf16* __restrict__ wt, int ldt)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= rows * cols) return;
   const int r = i / cols, c = i - r * cols;
   const bf16 b = __float2bfloat16_rn(p[i]);
   w[(size_t)r * ldw + c] = b;
   if (wt) wt[(size_t)c * ldt + r] = b;
}

int blocks(long long n, int t = 256) { return (int)((n + t - 1) / t); }

}  // namespace

struct hamstr_mlp {
   int Bmax = 0;
   cudaStream_t st = nullptr;
   std::vector<void*> owned;
   // FP32 master parameters, Adam moments, gradients (padded shapes)
   float *W1, *b1, *W2, *b2, *W3, *b3, *W4, *b4;
   float *mW1, *mb1, *mW2, *mb2, *mW3, *mb3, *mW4, *mb4;
   float *vW1, *vb1, *vW2, *vb2, *vW3, *vb3, *vW4, *vb4;
   float *gW1, *gb1, *gW2, *gb2, *gW3, *gb3, *gW4t, *gb4;
   // BF16 weights: W1 [256][64], W2/W3 [256][256] and transposes, W4 [16][256], W4t [256][64]
   bf16 *W1b, *W2b, *W2t, *W3b, *W3t, *W4b, *W4t;
   // activations and their gradients for Bmax rows
   bf16 *X, *Xt, *H1, *H1t, *H2, *H2t, *H3, *H3t, *dZ4, *dZ4t, *dZ3, *dZ3t, *dZ2, *dZ2t, *dZ1, *dZ1t;
   float *Z1, *Z2, *Z3, *Y, *T, *part;
   double* lpart;
   int* err;
   int splits_w = 1;   // split-K factor of the weight gradients

   template <typename T>
   int alloc(T** p, size_t n)
   {
      if (cudaMalloc((void**)p, (n ? n : 1) * sizeof(T)) != cudaSuccess) return HAMSTR_GPU_ERR_NOMEM;
      owned.push_back(*p);
      return cudaMemsetAsync(*p, 0, (n ? n : 1) * sizeof(T), st) == cudaSuccess ? HAMSTR_GPU_OK : HAMSTR_GPU_ERR_CUDA;
   }
};

namespace {

int cuda_ok(cudaError_t e, const char* what)
{
   if (e == cudaSuccess) return HAMSTR_GPU_OK;
   set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
   return HAMSTR_GPU_ERR_CUDA;
}

// BF16 copies of every weight from the FP32 masters
int refresh_bf16(hamstr_mlp* h)
{
   cast_kernel<<<blocks(W * KIN), 256, 0, h->st>>>(h->W1, W, KIN, h->W1b, KIN, nullptr, 0);
   cast_kernel<<<blocks(W * W), 256, 0, h->st>>>(h->W2, W, W, h->W2b, W, h->W2t, W);
   cast_kernel<<<blocks(W * W), 256, 0, h->st>>>(h->W3, W, W, h->W3b, W, h->W3t, W);
   cast_kernel<<<blocks(NOP * W), 256, 0, h->st>>>(h->W4, NOP, W, h->W4b, W, h->W4t, KOP);
   return cuda_ok(cudaGetLastError(), "mlp cast");
}

int gemm(hamstr_mlp* h, const bf16* A, const bf16* B, int M, int N, int K, int mode, float* C = nullptr,
         const float* bias = nullptr, float* Z = nullptr, const float* Zin = nullptr, bf16* H = nullptr,
         bf16* Ht = nullptr, int splits = 1, int n_out = 0)
{
   mlp::GemmArgs a;
   a.A = A;
   a.B = B;
   a.M = M;
   a.N = N;
   a.K = K;
   a.mode = mode;
   a.C = C;
   a.bias = bias;
   a.Z = Z;
   a.Zin = Zin;
   a.H = H;
   a.Ht = Ht;
   a.splits = splits;
   a.n_out = n_out;
   a.err = h->err;
   return mlp::gemm(a, h->st);
}

// forward pass of rows already gathered into X (B a multiple of 128)
int forward(hamstr_mlp* h, int B)
{
   int st;
   if ((st = gemm(h, h->X, h->W1b, B, W, KIN, mlp::EPI_HIDDEN, nullptr, h->b1, h->Z1, nullptr, h->H1, h->H1t))) return st;
   if ((st = gemm(h, h->H1, h->W2b, B, W, W, mlp::EPI_HIDDEN, nullptr, h->b2, h->Z2, nullptr, h->H2, h->H2t))) return st;
   if ((st = gemm(h, h->H2, h->W3b, B, W, W, mlp::EPI_HIDDEN, nullptr, h->b3, h->Z3, nullptr, h->H3, h->H3t))) return st;
   return gemm(h, h->H3, h->W4b, B, NOP, W, mlp::EPI_OUT, h->Y, h->b4, nullptr, nullptr, nullptr, nullptr, 1, NOUT);
}

// weight gradient dW [M][N] = A [M][B] * Bm [N][B]^T with split K
int wgrad(hamstr_mlp* h, const bf16* A, const bf16* Bm, int M, int N, int B, float* out)
{
   const int sp = mlp::gemm_splits(B, h->splits_w);
   int st = gemm(h, A, Bm, M, N, B, mlp::EPI_F32, h->part, nullptr, nullptr, nullptr, nullptr, nullptr, sp);
   if (st) return st;
   splitk_kernel<<<blocks(M * N), 256, 0, h->st>>>(h->part, sp, M * N, out);
   return cuda_ok(cudaGetLastError(), "mlp split-K reduction");
}

// backward pass after forward and loss: all parameter gradients
int backward(hamstr_mlp* h, int B)
{
   int st;
   // output layer: dW4^T [256][16] = H3^T dZ4^T^T, db4 from the loss partials
   if ((st = wgrad(h, h->H3t, h->dZ4t, W, NOP, B, h->gW4t))) return st;
   // dZ3 = (dZ4 W4) * GELU'(Z3)
   if ((st = gemm(h, h->dZ4, h->W4t, B, W, KOP, mlp::EPI_BWD, nullptr, nullptr, nullptr, h->Z3, h->dZ3, h->dZ3t)))
      return st;
   if ((st = wgrad(h, h->dZ3t, h->H2t, W, W, B, h->gW3))) return st;
   rowsum_kernel<<<W, 256, 0, h->st>>>(h->dZ3t, B, h->gb3);
   if ((st = gemm(h, h->dZ3, h->W3t, B, W, W, mlp::EPI_BWD, nullptr, nullptr, nullptr, h->Z2, h->dZ2, h->dZ2t)))
      return st;
   if ((st = wgrad(h, h->dZ2t, h->H1t, W, W, B, h->gW2))) return st;
   rowsum_kernel<<<W, 256, 0, h->st>>>(h->dZ2t, B, h->gb2);
   if ((st = gemm(h, h->dZ2, h->W2t, B, W, W, mlp::EPI_BWD, nullptr, nullptr, nullptr, h->Z1, h->dZ1, h->dZ1t)))
      return st;
   if ((st = wgrad(h, h->dZ1t, h->Xt, W, KIN, B, h->gW1))) return st;
   rowsum_kernel<<<W, 256, 0, h->st>>>(h->dZ1t, B, h->gb1);
   return cuda_ok(cudaGetLastError(), "mlp backward");
}

// loss and output gradients; loss (host) summed from block partials in order
int loss(hamstr_mlp* h, int B, int B_valid, double* loss_out)
{
   const int nb = blocks(B);
   loss_kernel<<<nb, 256, 0, h->st>>>(h->Y, h->T, B, B_valid, h->dZ4, h->dZ4t, h->lpart);
   int st = cuda_ok(cudaGetLastError(), "mlp loss");
   if (st) return st;
   std::vector<double> p(5 * (size_t)nb);
   if ((st = cuda_ok(cudaMemcpyAsync(p.data(), h->lpart, p.size() * sizeof(double), cudaMemcpyDeviceToHost, h->st),
                     "mlp loss copy")))
      return st;
   if ((st = cuda_ok(cudaStreamSynchronize(h->st), "mlp loss sync"))) return st;
   double l = 0.0, g[NOP] = {0.0};
   for (int b = 0; b < nb; b++) {
      l += p[5 * b];
      for (int k = 0; k < NOUT; k++) g[k] += p[5 * b + 1 + k];
   }
   float gb4[NOP];
   for (int k = 0; k < NOP; k++) gb4[k] = (float)g[k];
   if ((st = cuda_ok(cudaMemcpyAsync(h->gb4, gb4, sizeof(gb4), cudaMemcpyHostToDevice, h->st), "mlp db4"))) return st;
   if ((st = cuda_ok(cudaStreamSynchronize(h->st), "mlp db4 sync"))) return st;
   if (loss_out) *loss_out = l;
   return HAMSTR_GPU_OK;
}

int err_check(hamstr_mlp* h)
{
   int e = 0;
   int st = cuda_ok(cudaMemcpyAsync(&e, h->err, sizeof(int), cudaMemcpyDeviceToHost, h->st), "mlp error word");
   if (!st) st = cuda_ok(cudaStreamSynchronize(h->st), "mlp sync");
   if (st) return st;
   if (e) {
      set_last_error("mlp gemm: a tensor-core pipeline wait timed out");
      cudaMemsetAsync(h->err, 0, sizeof(int), h->st);
      return HAMSTR_GPU_ERR_CUDA;
   }
   return HAMSTR_GPU_OK;
}

// (pointer, rows, cols, padded leading dimension) of each logical tensor
struct View {
   float* p;
   int rows, cols, ld;
};

std::vector<View> views(hamstr_mlp* h, bool grads)
{
   if (!grads)
      return {{h->W1, W, NIN, KIN}, {h->b1, 1, W, W},    {h->W2, W, W, W}, {h->b2, 1, W, W},
              {h->W3, W, W, W},     {h->b3, 1, W, W},    {h->W4, NOUT, W, W}, {h->b4, 1, NOUT, NOP}};
   return {{h->gW1, W, NIN, KIN}, {h->gb1, 1, W, W},  {h->gW2, W, W, W}, {h->gb2, 1, W, W},
           {h->gW3, W, W, W},     {h->gb3, 1, W, W},  {nullptr, NOUT, W, 0}, {h->gb4, 1, NOUT, NOP}};
}

}  // namespace

extern "C" {

int hamstr_mlp_nparams(void) { return kNParams; }

int hamstr_mlp_set_params(hamstr_mlp* h, const float* params);

int hamstr_mlp_destroy(hamstr_mlp* h)
{
   if (!h) return HAMSTR_GPU_OK;
   if (h->st) cudaStreamSynchronize(h->st);
   for (void* p : h->owned) cudaFree(p);
   if (h->st) cudaStreamDestroy(h->st);
   delete h;
   return HAMSTR_GPU_OK;
}

int hamstr_mlp_create(int Bmax, unsigned long long seed, hamstr_mlp** out)
{
   if (!out || Bmax < 128) return HAMSTR_GPU_ERR_ARG;
   *out = nullptr;
   hamstr_mlp* h = new hamstr_mlp;
   h->Bmax = (Bmax + 127) / 128 * 128;
   if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) {
      delete h;
      return HAMSTR_GPU_ERR_CUDA;
   }
   const size_t B = h->Bmax;
   int st = HAMSTR_GPU_OK;
#define A(x, n) \
   if (!st) st = h->alloc(&h->x, (n))
   A(W1, W * KIN); A(b1, W); A(W2, W * W); A(b2, W); A(W3, W * W); A(b3, W); A(W4, NOP * W); A(b4, NOP);
   A(mW1, W * KIN); A(mb1, W); A(mW2, W * W); A(mb2, W); A(mW3, W * W); A(mb3, W); A(mW4, NOP * W); A(mb4, NOP);
   A(vW1, W * KIN); A(vb1, W); A(vW2, W * W); A(vb2, W); A(vW3, W * W); A(vb3, W); A(vW4, NOP * W); A(vb4, NOP);
   A(gW1, W * KIN); A(gb1, W); A(gW2, W * W); A(gb2, W); A(gW3, W * W); A(gb3, W); A(gW4t, W * NOP); A(gb4, NOP);
   A(W1b, W * KIN); A(W2b, W * W); A(W2t, W * W); A(W3b, W * W); A(W3t, W * W); A(W4b, NOP * W); A(W4t, W * KOP);
   A(X, B * KIN); A(Xt, B * KIN); A(H1, B * W); A(H1t, B * W); A(H2, B * W); A(H2t, B * W); A(H3, B * W);
   A(H3t, B * W); A(dZ4, B * KOP); A(dZ4t, B * NOP); A(dZ3, B * W); A(dZ3t, B * W); A(dZ2, B * W); A(dZ2t, B * W);
   A(dZ1, B * W); A(dZ1t, B * W);
   A(Z1, B * W); A(Z2, B * W); A(Z3, B * W); A(Y, B * NOUT); A(T, B * NOUT);
   A(lpart, 5 * ((B + 255) / 256));
   A(err, 1);
#undef A
   // split-K for the weight gradients: enough CTAs for the GPU (two
   // 128-row tiles of M per 256-wide N)
   int dev = 0, nsm = 148;
   cudaGetDevice(&dev);
   cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
   h->splits_w = std::max(1, nsm / 2);
   if (!st) st = h->alloc(&h->part, (size_t)mlp::gemm_splits((int)B, h->splits_w) * W * W);
   if (st) {
      hamstr_mlp_destroy(h);
      return st;
   }
   // initial weights: uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)), seeded,
   // biases zero (the common default for GELU MLPs)
   std::vector<float> p(kNParams, 0.f);
   unsigned long long s = seed ? seed : 1;
   auto rnd = [&]() {
      s ^= s << 13;
      s ^= s >> 7;
      s ^= s << 17;   // xorshift64 (Marsaglia, 2003)
      return (double)(s >> 11) * (1.0 / 9007199254740992.0);
   };
   size_t o = 0;
   const int fan[4] = {NIN, W, W, W}, rows[4] = {W, W, W, NOUT};
   for (int l = 0; l < 4; l++) {
      const double a = 1.0 / std::sqrt((double)fan[l]);
      for (int i = 0; i < rows[l] * fan[l]; i++) p[o++] = (float)((2.0 * rnd() - 1.0) * a);
      o += rows[l];
   }
   *out = h;
   st = hamstr_mlp_set_params(h, p.data());
   if (st) {
      hamstr_mlp_destroy(h);
      *out = nullptr;
   }
   return st;
}

int hamstr_mlp_set_params(hamstr_mlp* h, const float* params)
{
   if (!h || !params) return HAMSTR_GPU_ERR_ARG;
   size_t o = 0;
   for (const View& v : views(h, false)) {
      std::vector<float> buf((size_t)v.rows * v.ld, 0.f);
      for (int r = 0; r < v.rows; r++)
         for (int c = 0; c < v.cols; c++) buf[(size_t)r * v.ld + c] = params[o++];
      int st = cuda_ok(cudaMemcpyAsync(v.p, buf.data(), buf.size() * sizeof(float), cudaMemcpyHostToDevice, h->st),
                       "mlp set params");
      if (st) return st;
   }
   int st = refresh_bf16(h);
   if (st) return st;
   return cuda_ok(cudaStreamSynchronize(h->st), "mlp set params sync");
}

static int get_tensors(hamstr_mlp* h, bool grads, float* out)
{
   size_t o = 0;
   for (const View& v : views(h, grads)) {
      std::vector<float> buf;
      if (v.p) {
         buf.resize((size_t)v.rows * v.ld);
         int st = cuda_ok(cudaMemcpyAsync(buf.data(), v.p, buf.size() * sizeof(float), cudaMemcpyDeviceToHost, h->st),
                          "mlp get");
         if (!st) st = cuda_ok(cudaStreamSynchronize(h->st), "mlp get sync");
         if (st) return st;
         for (int r = 0; r < v.rows; r++)
            for (int c = 0; c < v.cols; c++) out[o++] = buf[(size_t)r * v.ld + c];
      } else {
         // dW4 is kept transposed ([256][16])
         buf.resize((size_t)W * NOP);
         int st = cuda_ok(cudaMemcpyAsync(buf.data(), h->gW4t, buf.size() * sizeof(float), cudaMemcpyDeviceToHost, h->st),
                          "mlp get");
         if (!st) st = cuda_ok(cudaStreamSynchronize(h->st), "mlp get sync");
         if (st) return st;
         for (int r = 0; r < NOUT; r++)
            for (int c = 0; c < W; c++) out[o++] = buf[(size_t)c * NOP + r];
      }
   }
   return HAMSTR_GPU_OK;
}

int hamstr_mlp_get_params(hamstr_mlp* h, float* out)
{
   if (!h || !out) return HAMSTR_GPU_ERR_ARG;
   return get_tensors(h, false, out);
}

int hamstr_mlp_get_grads(hamstr_mlp* h, float* out)
{
   if (!h || !out) return HAMSTR_GPU_ERR_ARG;
   return get_tensors(h, true, out);
}

int hamstr_mlp_forward(hamstr_mlp* h, const float* feat, int n, float* y)
{
   if (!h || !feat || !y || n < 1) return HAMSTR_GPU_ERR_ARG;
   for (int r0 = 0; r0 < n; r0 += h->Bmax) {
      const int nv = std::min(h->Bmax, n - r0);
      const int B = (nv + 127) / 128 * 128;
      gather_kernel<<<blocks(B), 256, 0, h->st>>>(feat + (size_t)r0 * NIN, nullptr, nv, B, nv, 0, 0, h->X, h->Xt,
                                                  nullptr);
      int st = cuda_ok(cudaGetLastError(), "mlp gather");
      if (!st) st = forward(h, B);
      if (!st)
         st = cuda_ok(cudaMemcpyAsync(y + (size_t)r0 * NOUT, h->Y, (size_t)nv * NOUT * sizeof(float),
                                      cudaMemcpyDeviceToDevice, h->st),
                      "mlp output");
      if (st) return st;
   }
   return err_check(h);
}

int hamstr_mlp_grad(hamstr_mlp* h, const float* feat, const float* targ, int n, double* loss_out)
{
   if (!h || !feat || !targ || n < 1 || n > h->Bmax) return HAMSTR_GPU_ERR_ARG;
   const int B = (n + 127) / 128 * 128;
   gather_kernel<<<blocks(B), 256, 0, h->st>>>(feat, targ, n, B, n, 0, 0, h->X, h->Xt, h->T);
   int st = cuda_ok(cudaGetLastError(), "mlp gather");
   if (!st) st = forward(h, B);
   if (!st) st = loss(h, B, n, loss_out);
   if (!st) st = backward(h, B);
   if (!st) st = err_check(h);
   return st;
}

int hamstr_mlp_train_step(hamstr_mlp* h, const float* feat_all, const float* targ_all, long long n_all, int batch,
                          unsigned long long seed, unsigned long long step, float lr, double* loss_out)
{
   if (!h || !feat_all || !targ_all || n_all < 1 || batch < 128 || batch > h->Bmax || batch % 128 || !seed)
      return HAMSTR_GPU_ERR_ARG;
   const int B = batch;
   gather_kernel<<<blocks(B), 256, 0, h->st>>>(feat_all, targ_all, n_all, B, B, seed, step, h->X, h->Xt, h->T);
   int st = cuda_ok(cudaGetLastError(), "mlp gather");
   if (!st) st = forward(h, B);
   if (!st) st = loss(h, B, B, loss_out);
   if (!st) st = backward(h, B);
   if (st) return st;
   // Adam, t = step + 1
   const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
   const float c1 = 1.f - std::pow(b1, (float)(step + 1)), c2 = 1.f - std::pow(b2, (float)(step + 1));
   adam_kernel<<<blocks(W * KIN), 256, 0, h->st>>>(h->W1, h->gW1, 0, h->mW1, h->vW1, W, KIN, lr, b1, b2, eps, c1, c2,
                                                   h->W1b, KIN, nullptr, 0);
   adam_kernel<<<blocks(W), 256, 0, h->st>>>(h->b1, h->gb1, 0, h->mb1, h->vb1, 1, W, lr, b1, b2, eps, c1, c2, nullptr,
                                             0, nullptr, 0);
   adam_kernel<<<blocks(W * W), 256, 0, h->st>>>(h->W2, h->gW2, 0, h->mW2, h->vW2, W, W, lr, b1, b2, eps, c1, c2,
                                                 h->W2b, W, h->W2t, W);
   adam_kernel<<<blocks(W), 256, 0, h->st>>>(h->b2, h->gb2, 0, h->mb2, h->vb2, 1, W, lr, b1, b2, eps, c1, c2, nullptr,
                                             0, nullptr, 0);
   adam_kernel<<<blocks(W * W), 256, 0, h->st>>>(h->W3, h->gW3, 0, h->mW3, h->vW3, W, W, lr, b1, b2, eps, c1, c2,
                                                 h->W3b, W, h->W3t, W);
   adam_kernel<<<blocks(W), 256, 0, h->st>>>(h->b3, h->gb3, 0, h->mb3, h->vb3, 1, W, lr, b1, b2, eps, c1, c2, nullptr,
                                             0, nullptr, 0);
   adam_kernel<<<blocks(NOP * W), 256, 0, h->st>>>(h->W4, h->gW4t, 1, h->mW4, h->vW4, NOP, W, lr, b1, b2, eps, c1, c2,
                                                   h->W4b, W, h->W4t, KOP);
   adam_kernel<<<blocks(NOP), 256, 0, h->st>>>(h->b4, h->gb4, 0, h->mb4, h->vb4, 1, NOP, lr, b1, b2, eps, c1, c2,
                                               nullptr, 0, nullptr, 0);
   st = cuda_ok(cudaGetLastError(), "mlp adam");
   if (!st) st = err_check(h);
   return st;
}

}  // extern "C"
