/*
 * mlp_oracle.c -- CPU restatement of the warm-start network (FP64).
 *
 * TEST INFRASTRUCTURE ONLY: the parity tests call it to check the
 * tensor-core forward and backward passes; the product never does.
 *
 * Network: 5 -> 256 -> 256 -> 256 -> 4, GELU(z) = z/2 (1 + erf(z/sqrt2))
 * on the hidden layers, loss = mean over rows and the 4 outputs of the
 * squared error.  With `bf16` set, the values the GPU path holds in BF16
 * are rounded the same way (round to nearest even): the inputs, the
 * weights, the hidden activations and the back-propagated dZ of every
 * layer; everything else is FP64 (the GPU accumulates in FP32).  Without
 * it this is the exact FP64 network, checked by finite differences.
 * Parameters: W1[256][5] b1 W2[256][256] b2 W3[256][256] b3 W4[4][256] b4.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NW 256
#define NIN 5
#define NOUT 4

int mo_nparams(void) { return NW * NIN + NW + 2 * (NW * NW + NW) + NOUT * NW + NOUT; }

static double bf16r(double x, int on)
{
   float f;
   unsigned int u;
   if (!on) return x;
   f = (float)x;
   memcpy(&u, &f, 4);
   if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x7fffu + ((u >> 16) & 1u)) & 0xffff0000u;
   memcpy(&f, &u, 4);
   return (double)f;
}

static double gelu(double z) { return 0.5 * z * (1.0 + erf(z / sqrt(2.0))); }
static double gelu_grad(double z)
{
   return 0.5 * (1.0 + erf(z / sqrt(2.0))) + z * exp(-0.5 * z * z) / sqrt(2.0 * 3.14159265358979323846);
}

/* out[n][r] = in[n][k] * W[r][k]^T + b[r] */
static void dense(const double* in, int n, int k, const double* Wt, const double* b, int r, double* out)
{
   int i, j, l;
   for (i = 0; i < n; i++)
      for (j = 0; j < r; j++) {
         double a = 0.0;
         for (l = 0; l < k; l++) a += in[(size_t)i * k + l] * Wt[(size_t)j * k + l];
         out[(size_t)i * r + j] = a + b[j];
      }
}

/* loss and gradient (grad may be NULL); y (may be NULL) receives the outputs */
double mo_loss_grad(const double* p, const double* feat, const double* targ, int n, int bf16, double* grad,
                    double* y)
{
   const int nl[4] = {NIN, NW, NW, NW}, nr[4] = {NW, NW, NW, NOUT};
   const double* Wl[4];
   const double* bl[4];
   double* Wq[4];
   double *act[4], *Z[3], *Y, *d, *dn;
   double loss = 0.0;
   size_t o = 0;
   int l, i, j, k;
   for (l = 0; l < 4; l++) {
      Wl[l] = p + o;
      o += (size_t)nl[l] * nr[l];
      bl[l] = p + o;
      o += nr[l];
      Wq[l] = (double*)malloc(sizeof(double) * nl[l] * nr[l]);
      for (i = 0; i < nl[l] * nr[l]; i++) Wq[l][i] = bf16r(Wl[l][i], bf16);
   }
   act[0] = (double*)malloc(sizeof(double) * n * NIN);
   for (i = 0; i < n * NIN; i++) act[0][i] = bf16r(feat[i], bf16);
   for (l = 0; l < 3; l++) {
      Z[l] = (double*)malloc(sizeof(double) * n * NW);
      act[l + 1] = (double*)malloc(sizeof(double) * n * NW);
      dense(act[l], n, nl[l], Wq[l], bl[l], NW, Z[l]);
      for (i = 0; i < n * NW; i++) act[l + 1][i] = bf16r(gelu(Z[l][i]), bf16);
   }
   Y = (double*)malloc(sizeof(double) * n * NOUT);
   dense(act[3], n, NW, Wq[3], bl[3], NOUT, Y);
   for (i = 0; i < n * NOUT; i++) loss += (Y[i] - targ[i]) * (Y[i] - targ[i]);
   loss /= (double)(n * NOUT);
   if (y) memcpy(y, Y, sizeof(double) * n * NOUT);
   if (grad) {
      /* walk back: d = dL/dZ of layer l (rows n, width nr[l]) */
      double* g = grad;
      size_t go[4], gb[4];
      o = 0;
      for (l = 0; l < 4; l++) {
         go[l] = o;
         o += (size_t)nl[l] * nr[l];
         gb[l] = o;
         o += nr[l];
      }
      d = (double*)malloc(sizeof(double) * n * NOUT);
      for (i = 0; i < n * NOUT; i++) d[i] = 2.0 * (Y[i] - targ[i]) / (double)(n * NOUT);
      /* the output bias takes the unrounded dY, as on the GPU */
      for (j = 0; j < NOUT; j++) {
         double s = 0.0;
         for (i = 0; i < n; i++) s += d[(size_t)i * NOUT + j];
         g[gb[3] + j] = s;
      }
      for (i = 0; i < n * NOUT; i++) d[i] = bf16r(d[i], bf16);
      for (l = 3; l >= 0; l--) {
         /* dW[r][k] = sum_i d[i][r] act[l][i][k] */
         for (j = 0; j < nr[l]; j++)
            for (k = 0; k < nl[l]; k++) {
               double s = 0.0;
               for (i = 0; i < n; i++) s += d[(size_t)i * nr[l] + j] * act[l][(size_t)i * nl[l] + k];
               g[go[l] + (size_t)j * nl[l] + k] = s;
            }
         if (l < 3) {
            for (j = 0; j < nr[l]; j++) {
               double s = 0.0;
               for (i = 0; i < n; i++) s += d[(size_t)i * nr[l] + j];
               g[gb[l] + j] = s;
            }
         }
         if (l == 0) break;
         /* dZ of layer l-1 = (d W_l) * GELU'(Z_{l-1}) */
         dn = (double*)malloc(sizeof(double) * n * NW);
         for (i = 0; i < n; i++)
            for (k = 0; k < NW; k++) {
               double s = 0.0;
               for (j = 0; j < nr[l]; j++) s += d[(size_t)i * nr[l] + j] * Wq[l][(size_t)j * nl[l] + k];
               dn[(size_t)i * NW + k] = bf16r(s * gelu_grad(Z[l - 1][(size_t)i * NW + k]), bf16);
            }
         free(d);
         d = dn;
      }
      free(d);
   }
   for (l = 0; l < 4; l++) {
      free(Wq[l]);
      free(act[l]);
   }
   for (l = 0; l < 3; l++) free(Z[l]);
   free(Y);
   return loss;
}
