// mdt_train_gemm.cu -- the network of a training step as BF16 GEMMs on the tensor cores
// (cuBLAS, BF16 operands, FP32 accumulation), for networks with two hidden layers of at
// most 32 nodes and at most 48 descriptors per element.
//
// The training kernel (mdt_train.cu) keeps the descriptor work: forces by the descriptor
// VJP, the loss and its adjoints, and the descriptor JVP along them.  What it does per atom
// with lanes = nodes is done here over all atoms of the step's configurations at once,
// rows = atoms ordered by element (one row block per element, so every product is a plain
// GEMM with that element's weights):
//   forward   z1 = x W1 + b1, h1 = f1(z1), z2 = h1 W2 + b2, h2 = f2(z2), z3 = h2.w3 + b3
//   backward  dl3 = f3'(z3), dl2 = f2'(z2) w3 dl3, dl1 = f1'(z1) (dl2 W2^T), dE/dx = dl1 W1^T
//   tangent   (x' from the JVP)  zd1 = x' W1, hd1 = f1'(z1) zd1, zd2 = hd1 W2, hd2 = f2'(z2) zd2
//   second    dp3 = f3''(z3) (hd2.w3), dp2 = f2'(z2) w3 dp3 + f2''(z2) zd2 w3 dl3,
//             dp1 = f1'(z1) (dp2 W2^T) + f1''(z1) zd1 (dl2 W2^T)
//   gradient  dW_l = (a h_(l-1) + hd_(l-1))^T dl_l + h_(l-1)^T dp_l,  db_l = sum (a dl_l + dp_l)
// (a: dL/dE of the row's configuration), the forward-over-reverse sweep of the training
// kernel written as products over rows.  The weight-gradient products sum over atoms
// (K = rows).  Results land in the same FP64 gradient array as the kernel's own sweep.
// Split mode (BF16X3) stores every operand as a BF16 high part and the BF16 rounding of the
// residual (at T.lo elements further on) and forms each product as hi*hi + hi*lo + lo*hi:
// about 16 significant bits, as the tensor-core inference does.  Plain BF16 rounds the
// forward sums by ~2^-9, which for a trained network is ~10 meV per atom of energy -- more
// than its true energy error, so the energy term of the loss gradient is then rounding.
#include <cublas_v2.h>
#include <cuda_bf16.h>

#include <algorithm>

#include "mdt_internal.h"
#include "mdt_nn.cuh"

namespace mdt {

namespace {

constexpr int kIn = 48;   // row width of descriptor arrays (inputs padded)
constexpr int kHid = 32;  // row width of hidden-layer arrays

__device__ __forceinline__ uint8_t act_of(const NNDev &M, int e, int l, int n) {
    return M.act[(e * kMaxLayers + (l - 1)) * kMaxNodes + n];
}

__device__ __forceinline__ int elem_of_row(const GemmTrain &T, int r) { return r < T.rows[1] ? 0 : 1; }

// a BF16 operand value; in split mode also its residual in the low part
__device__ __forceinline__ void st_op(const GemmTrain &T, __nv_bfloat16 *p, size_t k, float v) {
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    p[k] = h;
    if (T.split) p[k + T.lo] = __float2bfloat16_rn(v - __bfloat162float(h));
}

// weights of both elements as BF16 row-major blocks: W1 [kIn x kHid], W2 [kHid x kHid]
__global__ void weights_bf16(GemmTrain T) {
    const NNDev &M = T.M;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 2 * (kIn + kHid) * kHid; k += gridDim.x * blockDim.x) {
        const int e = k / ((kIn + kHid) * kHid), q = k % ((kIn + kHid) * kHid);
        float v = 0.f;
        if (e < M.nelem) {
            const float *we = T.theta + (size_t)e * M.maxweights;
            if (q < kIn * kHid) {
                const int p = q / kHid, n = q % kHid, n1 = M.nodes[e][1];
                if (p < M.nodes[e][0] && n < n1) v = we[M.woff[e][1] + p * n1 + n];
            } else {
                const int p = (q - kIn * kHid) / kHid, n = (q - kIn * kHid) % kHid, n1 = M.nodes[e][1],
                          n2 = M.nodes[e][2];
                if (p < n1 && n < n2) v = we[M.woff[e][2] + p * n2 + n];
            }
        }
        st_op(T, T.w, k, v);
    }
}

// scaled descriptors of every row (getshortatomic.f90:174-236 scaling)
__global__ void gather_x(GemmTrain T) {
    const NNDev &M = T.M;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < T.R; r += gridDim.x * blockDim.x) {
        const int e = elem_of_row(T, r), sl = T.slot[r];
        for (int s = 0; s < kIn; ++s) {
            float v = 0.f;
            if (s < M.nsf[e]) {
                const double mn = M.smin[e * M.maxsf + s], w = M.smax[e * M.maxsf + s] - mn;
                v = (float)((T.G[(size_t)sl * M.maxsf + s] - mn) / w * (M.scmax - M.scmin) + M.scmin);
            }
            T.f.x[(size_t)r * kIn + s] = v;
            st_op(T, T.b.x, (size_t)r * kIn + s, v);
        }
    }
}

__global__ void after_f1(GemmTrain T) {  // z1 += b1; h1 = f1(z1)
    const NNDev &M = T.M;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < T.R; r += gridDim.x * blockDim.x) {
        const int e = elem_of_row(T, r), n1 = M.nodes[e][1], n0 = M.nodes[e][0];
        const float *b1 = T.theta + (size_t)e * M.maxweights + M.woff[e][1] + n0 * n1;
        for (int n = 0; n < kHid; ++n) {
            const size_t k = (size_t)r * kHid + n;
            float z = 0.f, h = 0.f;
            if (n < n1) {
                z = T.f.z1[k] + b1[n];
                h = act_fn<float>(act_of(M, e, 1, n), z);
            }
            T.f.z1[k] = z;
            T.f.h1[k] = h;
            st_op(T, T.b.h1, k, h);
        }
    }
}

__global__ void after_f2(GemmTrain T) {  // z2 += b2; h2, z3, output, dl3, dl2
    const NNDev &M = T.M;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < T.R; r += gridDim.x * blockDim.x) {
        const int e = elem_of_row(T, r), n1 = M.nodes[e][1], n2 = M.nodes[e][2];
        const float *we = T.theta + (size_t)e * M.maxweights;
        const float *b2 = we + M.woff[e][2] + n1 * n2, *w3 = we + M.woff[e][3];
        float z3 = w3[n2];
        for (int n = 0; n < n2; ++n) {
            const size_t k = (size_t)r * kHid + n;
            const float z = T.f.z2[k] + b2[n];
            const float h = act_fn<float>(act_of(M, e, 2, n), z);
            T.f.z2[k] = z;
            T.f.h2[k] = h;
            z3 += w3[n] * h;
        }
        const uint8_t a3 = act_of(M, e, 3, 0);
        const float out = act_fn<float>(a3, z3), dl3 = act_dfn<float>(a3, z3, out);
        T.z3[r] = z3;
        T.out[r] = out;
        T.dl3[r] = dl3;
        T.eat[T.slot[r]] = (double)out;
        for (int n = 0; n < kHid; ++n) {
            const size_t k = (size_t)r * kHid + n;
            float d = 0.f;
            if (n < n2) d = act_dfn<float>(act_of(M, e, 2, n), T.f.z2[k], T.f.h2[k]) * w3[n] * dl3;
            T.f.dl2[k] = d;
            st_op(T, T.b.dl2, k, d);
        }
    }
}

__global__ void after_b1(GemmTrain T) {  // s2 = dl2 W2^T (in f.s2); dl1 = f1'(z1) s2
    const NNDev &M = T.M;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < T.R; r += gridDim.x * blockDim.x) {
        const int e = elem_of_row(T, r), n1 = M.nodes[e][1];
        for (int n = 0; n < kHid; ++n) {
            const size_t k = (size_t)r * kHid + n;
            float d = 0.f;
            if (n < n1) d = act_dfn<float>(act_of(M, e, 1, n), T.f.z1[k], T.f.h1[k]) * T.f.s2[k];
            T.f.dl1[k] = d;
            st_op(T, T.b.dl1, k, d);
        }
    }
}

__global__ void after_b0(GemmTrain T) {  // dE/dG = (dl1 W1^T) dscale -> dg of the row's slot
    const NNDev &M = T.M;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < T.R; r += gridDim.x * blockDim.x) {
        const int e = elem_of_row(T, r), sl = T.slot[r];
        for (int s = 0; s < M.nsf[e]; ++s) {
            const double w = M.smax[e * M.maxsf + s] - M.smin[e * M.maxsf + s];
            T.dg[(size_t)sl * M.maxsf + s] = T.f.cv[(size_t)r * kIn + s] * (float)((M.scmax - M.scmin) / w);
        }
    }
}

__global__ void gather_xd(GemmTrain T) {  // x' and a x + x' of every row
    const NNDev &M = T.M;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < T.R; r += gridDim.x * blockDim.x) {
        const int e = elem_of_row(T, r), sl = T.slot[r];
        const float a = (float)T.arow[sl];
        T.a[r] = a;
        for (int s = 0; s < kIn; ++s) {
            const float xd = s < M.nsf[e] ? T.xdot[(size_t)sl * M.maxsf + s] : 0.f;
            const size_t k = (size_t)r * kIn + s;
            st_op(T, T.b.xd, k, xd);
            st_op(T, T.b.ax, k, a * T.f.x[k] + xd);
        }
    }
}

__global__ void after_t1(GemmTrain T) {  // zd1 = x' W1 (in f.zd1); hd1 = f1'(z1) zd1; a h1 + hd1
    const NNDev &M = T.M;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < T.R; r += gridDim.x * blockDim.x) {
        const int e = elem_of_row(T, r), n1 = M.nodes[e][1];
        const float a = T.a[r];
        for (int n = 0; n < kHid; ++n) {
            const size_t k = (size_t)r * kHid + n;
            float hd = 0.f;
            if (n < n1) hd = act_dfn<float>(act_of(M, e, 1, n), T.f.z1[k], T.f.h1[k]) * T.f.zd1[k];
            st_op(T, T.b.hd1, k, hd);
            st_op(T, T.b.ah1, k, a * T.f.h1[k] + hd);
        }
    }
}

// output layer and layer-2 bias gradients of a block's rows: summed per element in shared
// memory, then one FP64 atomic per weight
__global__ void after_t2(GemmTrain T) {  // zd2 = hd1 W2 (in f.zd2); dp2; dw3, db3, db2
    const NNDev &M = T.M;
    __shared__ float acc[2][2 * kHid + 1];
    for (int k = threadIdx.x; k < 2 * (2 * kHid + 1); k += blockDim.x) (&acc[0][0])[k] = 0.f;
    __syncthreads();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < T.R; r += gridDim.x * blockDim.x) {
        const int e = elem_of_row(T, r), n1 = M.nodes[e][1], n2 = M.nodes[e][2];
        const float *w3 = T.theta + (size_t)e * M.maxweights + M.woff[e][3];
        const float a = T.a[r], dl3 = T.dl3[r];
        float zd3 = 0.f;
        float hd2[kHid];
        for (int n = 0; n < kHid; ++n) {
            const size_t k = (size_t)r * kHid + n;
            hd2[n] = n < n2 ? act_dfn<float>(act_of(M, e, 2, n), T.f.z2[k], T.f.h2[k]) * T.f.zd2[k] : 0.f;
            zd3 += n < n2 ? w3[n] * hd2[n] : 0.f;
        }
        const uint8_t a3 = act_of(M, e, 3, 0);
        const float dp3 = act_ddfn<float>(a3, T.z3[r], T.out[r]) * zd3;
        for (int n = 0; n < kHid; ++n) {
            const size_t k = (size_t)r * kHid + n;
            float dp = 0.f;
            if (n < n2) {
                const uint8_t ac = act_of(M, e, 2, n);
                dp = act_dfn<float>(ac, T.f.z2[k], T.f.h2[k]) * w3[n] * dp3 +
                     act_ddfn<float>(ac, T.f.z2[k], T.f.h2[k]) * T.f.zd2[k] * w3[n] * dl3;
                atomicAdd(&acc[e][n], dl3 * (a * T.f.h2[k] + hd2[n]) + dp3 * T.f.h2[k]);  // w3
                atomicAdd(&acc[e][kHid + n], a * T.f.dl2[k] + dp);                       // b2
            }
            st_op(T, T.b.dp2, k, dp);
        }
        atomicAdd(&acc[e][2 * kHid], a * dl3 + dp3);  // b3
        (void)n1;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * (2 * kHid + 1); k += blockDim.x) {
        const int e = k / (2 * kHid + 1), q = k % (2 * kHid + 1);
        if (e >= M.nelem) continue;
        const int n1 = M.nodes[e][1], n2 = M.nodes[e][2];
        double *g = T.grad + (size_t)e * M.maxweights;
        const float v = acc[e][q];
        if (v == 0.f) continue;
        if (q < kHid) {
            if (q < n2) atomicAdd(&g[M.woff[e][3] + q], (double)v);
        } else if (q < 2 * kHid) {
            if (q - kHid < n2) atomicAdd(&g[M.woff[e][2] + n1 * n2 + (q - kHid)], (double)v);
        } else {
            atomicAdd(&g[M.woff[e][3] + n2], (double)v);
        }
    }
}

__global__ void after_s1(GemmTrain T) {  // sp2 = dp2 W2^T (in f.zd2's place: f.sp2); dp1; db1
    const NNDev &M = T.M;
    __shared__ float acc[2][kHid];
    for (int k = threadIdx.x; k < 2 * kHid; k += blockDim.x) (&acc[0][0])[k] = 0.f;
    __syncthreads();
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < T.R; r += gridDim.x * blockDim.x) {
        const int e = elem_of_row(T, r), n1 = M.nodes[e][1];
        const float a = T.a[r];
        for (int n = 0; n < kHid; ++n) {
            const size_t k = (size_t)r * kHid + n;
            float dp = 0.f;
            if (n < n1) {
                const uint8_t ac = act_of(M, e, 1, n);
                dp = act_dfn<float>(ac, T.f.z1[k], T.f.h1[k]) * T.f.sp2[k] +
                     act_ddfn<float>(ac, T.f.z1[k], T.f.h1[k]) * T.f.zd1[k] * T.f.s2[k];
                atomicAdd(&acc[e][n], a * T.f.dl1[k] + dp);
            }
            st_op(T, T.b.dp1, k, dp);
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < 2 * kHid; k += blockDim.x) {
        const int e = k / kHid, n = k % kHid;
        if (e >= M.nelem || n >= M.nodes[e][1] || acc[e][n] == 0.f) continue;
        const int n0 = M.nodes[e][0], n1 = M.nodes[e][1];
        atomicAdd(&T.grad[(size_t)e * M.maxweights + M.woff[e][1] + n0 * n1 + n], (double)acc[e][n]);
    }
}

__global__ void add_weight_grads(GemmTrain T) {  // gW1, gW2 of both elements into the gradient
    const NNDev &M = T.M;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 2 * (kIn + kHid) * kHid; k += gridDim.x * blockDim.x) {
        const int e = k / ((kIn + kHid) * kHid), q = k % ((kIn + kHid) * kHid);
        if (e >= M.nelem) continue;
        double *g = T.grad + (size_t)e * M.maxweights;
        const float v = T.gw[k];
        const int n1 = M.nodes[e][1], n2 = M.nodes[e][2];
        if (q < kIn * kHid) {
            const int p = q / kHid, n = q % kHid;
            if (p < M.nodes[e][0] && n < n1) g[M.woff[e][1] + p * n1 + n] += (double)v;
        } else {
            const int p = (q - kIn * kHid) / kHid, n = (q - kIn * kHid) % kHid;
            if (p < n1 && n < n2) g[M.woff[e][2] + p * n2 + n] += (double)v;
        }
    }
}

// C[R x N] (+)= A[R x K] B[K x N] (row-major; opB: B stored [N x K], i.e. A B^T)
cublasStatus_t rows_gemm(cublasHandle_t h, int R, int N, int K, const __nv_bfloat16 *A, int lda,
                         const __nv_bfloat16 *B, int ldb, bool transB, float *C, int ldc, float beta) {
    const float one = 1.f;
    return cublasGemmEx(h, transB ? CUBLAS_OP_T : CUBLAS_OP_N, CUBLAS_OP_N, N, R, K, &one, B, CUDA_R_16BF, ldb, A,
                        CUDA_R_16BF, lda, &beta, C, CUDA_R_32F, ldc, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
}
// C[K x N] (+)= A[R x K]^T B[R x N] (row-major; the sum runs over the R rows)
cublasStatus_t grad_gemm(cublasHandle_t h, int R, int K, int N, const __nv_bfloat16 *A, int lda,
                         const __nv_bfloat16 *B, int ldb, float *C, int ldc, float beta) {
    const float one = 1.f;
    return cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_T, N, K, R, &one, B, CUDA_R_16BF, ldb, A, CUDA_R_16BF, lda, &beta,
                        C, CUDA_R_32F, ldc, CUBLAS_COMPUTE_32F, CUBLAS_GEMM_DEFAULT);
}

// split-aware products: C (+)= A B as hi*hi (+ hi*lo + lo*hi)
bool rows_gemm3(const GemmTrain &T, cublasHandle_t h, int R, int N, int K, const __nv_bfloat16 *A, int lda,
                const __nv_bfloat16 *B, int ldb, bool transB, float *C, int ldc, float beta) {
    if (rows_gemm(h, R, N, K, A, lda, B, ldb, transB, C, ldc, beta) != CUBLAS_STATUS_SUCCESS) return false;
    if (!T.split) return true;
    return rows_gemm(h, R, N, K, A, lda, B + T.lo, ldb, transB, C, ldc, 1.f) == CUBLAS_STATUS_SUCCESS &&
           rows_gemm(h, R, N, K, A + T.lo, lda, B, ldb, transB, C, ldc, 1.f) == CUBLAS_STATUS_SUCCESS;
}
bool grad_gemm3(const GemmTrain &T, cublasHandle_t h, int R, int K, int N, const __nv_bfloat16 *A, int lda,
                const __nv_bfloat16 *B, int ldb, float *C, int ldc, float beta) {
    if (grad_gemm(h, R, K, N, A, lda, B, ldb, C, ldc, beta) != CUBLAS_STATUS_SUCCESS) return false;
    if (!T.split) return true;
    return grad_gemm(h, R, K, N, A, lda, B + T.lo, ldb, C, ldc, 1.f) == CUBLAS_STATUS_SUCCESS &&
           grad_gemm(h, R, K, N, A + T.lo, lda, B, ldb, C, ldc, 1.f) == CUBLAS_STATUS_SUCCESS;
}

int grid_of(int R) { return std::max(1, std::min(4096, (R + 255) / 256)); }

}  // namespace

size_t gemm_train_floats(int R) { return (size_t)R * (2 * kIn + 10 * kHid + 4); }
size_t gemm_train_bf16(int R) { return (size_t)R * (3 * kIn + 7 * kHid) + 2 * (size_t)(kIn + kHid) * kHid; }
size_t gemm_train_gw(int) { return 2 * (size_t)(kIn + kHid) * kHid; }

// carve the pools of GemmTrain (row arrays of R rows)
void gemm_train_carve(GemmTrain &T, float *fpool, __nv_bfloat16 *bpool, float *gw, int R) {
    const size_t Rz = (size_t)R;
    float *f = fpool;
    T.f.x = f; f += Rz * kIn;
    T.f.cv = f; f += Rz * kIn;
    T.f.z1 = f; f += Rz * kHid;
    T.f.h1 = f; f += Rz * kHid;
    T.f.z2 = f; f += Rz * kHid;
    T.f.h2 = f; f += Rz * kHid;
    T.f.dl1 = f; f += Rz * kHid;
    T.f.dl2 = f; f += Rz * kHid;
    T.f.s2 = f; f += Rz * kHid;
    T.f.zd1 = f; f += Rz * kHid;
    T.f.zd2 = f; f += Rz * kHid;
    T.f.sp2 = f; f += Rz * kHid;
    T.z3 = f; f += Rz;
    T.out = f; f += Rz;
    T.dl3 = f; f += Rz;
    T.a = f; f += Rz;
    __nv_bfloat16 *b = bpool;
    T.b.x = b; b += Rz * kIn;
    T.b.xd = b; b += Rz * kIn;
    T.b.ax = b; b += Rz * kIn;
    T.b.h1 = b; b += Rz * kHid;
    T.b.hd1 = b; b += Rz * kHid;
    T.b.ah1 = b; b += Rz * kHid;
    T.b.dl1 = b; b += Rz * kHid;
    T.b.dl2 = b; b += Rz * kHid;
    T.b.dp1 = b; b += Rz * kHid;
    T.b.dp2 = b; b += Rz * kHid;
    T.w = b;
    T.gw = gw;
    T.lo = gemm_train_bf16(R);
}

// forward and backward products: atomic outputs to eat, dE/dG to dg (for the training
// kernel's forces)
int gemm_train_forward(cublasHandle_t h, cudaStream_t s, const GemmTrain &T) {
    cublasSetStream(h, s);
    weights_bf16<<<64, 256, 0, s>>>(T);
    gather_x<<<grid_of(T.R), 256, 0, s>>>(T);
    for (int e = 0; e < T.M.nelem; ++e) {
        const int r0 = T.rows[e], R = T.rows[e + 1] - r0;
        if (R <= 0) continue;
        const int n0 = T.M.nodes[e][0], n1 = T.M.nodes[e][1];
        const __nv_bfloat16 *W1 = T.w + (size_t)e * (kIn + kHid) * kHid;
        if (!rows_gemm3(T, h, R, n1, n0, T.b.x + (size_t)r0 * kIn, kIn, W1, kHid, false, T.f.z1 + (size_t)r0 * kHid, kHid,
                      0.f) )
            return 1;
    }
    after_f1<<<grid_of(T.R), 256, 0, s>>>(T);
    for (int e = 0; e < T.M.nelem; ++e) {
        const int r0 = T.rows[e], R = T.rows[e + 1] - r0;
        if (R <= 0) continue;
        const int n1 = T.M.nodes[e][1], n2 = T.M.nodes[e][2];
        const __nv_bfloat16 *W2 = T.w + (size_t)e * (kIn + kHid) * kHid + kIn * kHid;
        if (!rows_gemm3(T, h, R, n2, n1, T.b.h1 + (size_t)r0 * kHid, kHid, W2, kHid, false, T.f.z2 + (size_t)r0 * kHid, kHid,
                      0.f) )
            return 1;
    }
    after_f2<<<grid_of(T.R), 256, 0, s>>>(T);
    for (int e = 0; e < T.M.nelem; ++e) {  // s2 = dl2 W2^T
        const int r0 = T.rows[e], R = T.rows[e + 1] - r0;
        if (R <= 0) continue;
        const int n1 = T.M.nodes[e][1], n2 = T.M.nodes[e][2];
        const __nv_bfloat16 *W2 = T.w + (size_t)e * (kIn + kHid) * kHid + kIn * kHid;
        if (!rows_gemm3(T, h, R, n1, n2, T.b.dl2 + (size_t)r0 * kHid, kHid, W2, kHid, true, T.f.s2 + (size_t)r0 * kHid, kHid,
                      0.f) )
            return 1;
    }
    after_b1<<<grid_of(T.R), 256, 0, s>>>(T);
    for (int e = 0; e < T.M.nelem; ++e) {  // dE/dx = dl1 W1^T
        const int r0 = T.rows[e], R = T.rows[e + 1] - r0;
        if (R <= 0) continue;
        const int n0 = T.M.nodes[e][0], n1 = T.M.nodes[e][1];
        const __nv_bfloat16 *W1 = T.w + (size_t)e * (kIn + kHid) * kHid;
        if (!rows_gemm3(T, h, R, n0, n1, T.b.dl1 + (size_t)r0 * kHid, kHid, W1, kHid, true, T.f.cv + (size_t)r0 * kIn, kIn,
                      0.f) )
            return 1;
    }
    after_b0<<<grid_of(T.R), 256, 0, s>>>(T);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

// tangent, second-order products and weight gradients into T.grad
int gemm_train_backward(cublasHandle_t h, cudaStream_t s, const GemmTrain &T) {
    cublasSetStream(h, s);
    gather_xd<<<grid_of(T.R), 256, 0, s>>>(T);
    for (int e = 0; e < T.M.nelem; ++e) {  // zd1 = x' W1
        const int r0 = T.rows[e], R = T.rows[e + 1] - r0;
        if (R <= 0) continue;
        const int n0 = T.M.nodes[e][0], n1 = T.M.nodes[e][1];
        const __nv_bfloat16 *W1 = T.w + (size_t)e * (kIn + kHid) * kHid;
        if (!rows_gemm3(T, h, R, n1, n0, T.b.xd + (size_t)r0 * kIn, kIn, W1, kHid, false, T.f.zd1 + (size_t)r0 * kHid, kHid,
                      0.f) )
            return 1;
    }
    after_t1<<<grid_of(T.R), 256, 0, s>>>(T);
    for (int e = 0; e < T.M.nelem; ++e) {  // zd2 = hd1 W2
        const int r0 = T.rows[e], R = T.rows[e + 1] - r0;
        if (R <= 0) continue;
        const int n1 = T.M.nodes[e][1], n2 = T.M.nodes[e][2];
        const __nv_bfloat16 *W2 = T.w + (size_t)e * (kIn + kHid) * kHid + kIn * kHid;
        if (!rows_gemm3(T, h, R, n2, n1, T.b.hd1 + (size_t)r0 * kHid, kHid, W2, kHid, false, T.f.zd2 + (size_t)r0 * kHid,
                      kHid, 0.f) )
            return 1;
    }
    after_t2<<<grid_of(T.R), 256, 0, s>>>(T);
    for (int e = 0; e < T.M.nelem; ++e) {  // sp2 = dp2 W2^T
        const int r0 = T.rows[e], R = T.rows[e + 1] - r0;
        if (R <= 0) continue;
        const int n1 = T.M.nodes[e][1], n2 = T.M.nodes[e][2];
        const __nv_bfloat16 *W2 = T.w + (size_t)e * (kIn + kHid) * kHid + kIn * kHid;
        if (!rows_gemm3(T, h, R, n1, n2, T.b.dp2 + (size_t)r0 * kHid, kHid, W2, kHid, true, T.f.sp2 + (size_t)r0 * kHid,
                      kHid, 0.f) )
            return 1;
    }
    after_s1<<<grid_of(T.R), 256, 0, s>>>(T);
    for (int e = 0; e < T.M.nelem; ++e) {  // weight gradients: sums over the element's rows
        const int r0 = T.rows[e], R = T.rows[e + 1] - r0;
        float *g1 = T.gw + (size_t)e * (kIn + kHid) * kHid, *g2 = g1 + kIn * kHid;
        if (R <= 0) {
            cudaMemsetAsync(g1, 0, sizeof(float) * (kIn + kHid) * kHid, s);
            continue;
        }
        const int n0 = T.M.nodes[e][0], n1 = T.M.nodes[e][1], n2 = T.M.nodes[e][2];
        if (!grad_gemm3(T, h, R, n0, n1, T.b.ax + (size_t)r0 * kIn, kIn, T.b.dl1 + (size_t)r0 * kHid, kHid, g1, kHid, 0.f) ||
            !grad_gemm3(T, h, R, n0, n1, T.b.x + (size_t)r0 * kIn, kIn, T.b.dp1 + (size_t)r0 * kHid, kHid, g1, kHid, 1.f) ||
            !grad_gemm3(T, h, R, n1, n2, T.b.ah1 + (size_t)r0 * kHid, kHid, T.b.dl2 + (size_t)r0 * kHid, kHid, g2, kHid,
                        0.f) ||
            !grad_gemm3(T, h, R, n1, n2, T.b.h1 + (size_t)r0 * kHid, kHid, T.b.dp2 + (size_t)r0 * kHid, kHid, g2, kHid,
                        1.f))
            return 1;
    }
    add_weight_grads<<<64, 256, 0, s>>>(T);
    return cudaGetLastError() == cudaSuccess ? 0 : 2;
}

}  // namespace mdt
