// Split-precision tensor-core axis passes (fft_split.cuh): the kernel and its
// instantiations for FP32 lines of 256, 512 and 1024 points.
//
// A 256-thread CTA owns L lines (4 contiguous, 8 strided) and one padded
// shared-memory buffer, used in place:
//   stage 1 (radix 16, tensor cores): every lane loads its MMA inputs straight
//     from global memory (c2r: from the staged half spectra), transforms its
//     warp's groups and writes the outputs to the buffer;
//   stage 2 (radix 16, tensor cores): every lane reads and twiddles all the
//     inputs of its warp's groups, the CTA synchronises, then transforms and
//     writes in place (for 256 points: stores to global memory instead);
//   stage 3 (radix 2 or 4 for 512 / 1024 points, CUDA cores): reads, twiddles,
//     transforms and stores to global memory;
//   r2c: the last stage writes the pair slots of the half-spectrum split.
#include "fft_split.cuh"

namespace gbfft {

namespace {

using namespace dev;
using split::kThreads;

template <int KIND, bool CONTIG, int N>
__global__ void __launch_bounds__(kThreads, 2) split_pass_kernel(const __grid_constant__ PassArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* S = reinterpret_cast<float2*>(smem_raw);
  using Ctx = LineCtx<float, KIND, CONTIG>;
  constexpr int L = CONTIG ? 4 : 8;                // lines a CTA (split_lines_per_cta)
  constexpr int TPL = kThreads / L;                // threads a line, standard mapping
  constexpr int NB = N / 16;                       // radix-16 butterflies a line
  constexpr int GPW = CONTIG ? NB / 16 : NB / 8;   // groups of 8 butterflies a warp
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, g = lane >> 2, q = lane & 3;
  const long long tile0 = (long long)blockIdx.x * L;
  const long long v = CONTIG ? 0 : (long long)blockIdx.y;

  // standard mapping (c2r staging, radix-2/4 stage, r2c split):
  // contiguous: TPL threads a line; strided: the lanes run across lines
  const int sline = CONTIG ? tid / TPL : tid % L;
  const int st = CONTIG ? tid % TPL : tid / L;
  Ctx cs;
  cs.init_at(a, st, sline, tile0 + sline, v, a.nlines);
  cs.tpl = TPL;
  // MMA mapping: contiguous, warps 2l and 2l+1 take line l, column g is
  // butterfly 8 j' + g of it; strided, column g is line g
  const int mline = CONTIG ? (w >> 1) : g;
  Ctx cm;
  cm.init_at(a, 0, mline, tile0 + mline, v, a.nlines);
  auto bfly = [&](int j) { return CONTIG ? (((w & 1) * GPW + j) * 8 + g) : (w + 8 * j); };
  // output column c of group j: its butterfly and its line
  auto obfly = [&](int j, int c) { return CONTIG ? (((w & 1) * GPW + j) * 8 + c) : (w + 8 * j); };
  auto oline = [&](int c) { return CONTIG ? mline : c; };

  split::DftFrag F;
  split::dft16_frag(F, lane);
  const int kk[4] = {2 * q, 2 * q + 1, 2 * q + 8, 2 * q + 9};
  float2 X[GPW][4];

  // ---- stage 1: radix 16, NS = 1 ------------------------------------------
  if constexpr (KIND == K_C2R) {
    cs.template stage_c2r<N, TPL>(S);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < GPW; ++j)
#pragma unroll
      for (int i = 0; i < 4; ++i) X[j][i] = cm.sgather_c2r(S, bfly(j) + kk[i] * NB);
    __syncthreads();
  } else {
#pragma unroll
    for (int j = 0; j < GPW; ++j)
#pragma unroll
      for (int i = 0; i < 4; ++i) X[j][i] = cm.gload(bfly(j) + kk[i] * NB);
  }
#pragma unroll
  for (int j = 0; j < GPW; ++j) {
    float2 y[4];
    split::mma_group(F, X[j], y, lane);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = i < 2 ? g : g + 8, c = 2 * q + (i & 1);
      S[cm.sidx_at(oline(c), obfly(j, c) * 16 + r)] = y[i];
    }
  }
  __syncthreads();

  // ---- stage 2: radix 16, NS = 16 -------------------------------------------
#pragma unroll
  for (int j = 0; j < GPW; ++j) {
    const int b = bfly(j), kb = b & 15;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      X[j][i] = S[cm.sidx(b + kk[i] * NB)];
      if (kk[i] > 0) X[j][i] = cmul(X[j][i], cm.twiddle(15 + (kk[i] - 1) * 16 + kb));
    }
  }
  __syncthreads();  // every input read before the buffer is overwritten
  if constexpr (N == 256) {
    // last stage: outputs to global memory (r2c: to the pair slots)
    Ctx c0 = cm, c1 = cm;
    if (!CONTIG) {
      c0.init_at(a, 0, 2 * q, tile0 + 2 * q, v, a.nlines);
      c1.init_at(a, 0, 2 * q + 1, tile0 + 2 * q + 1, v, a.nlines);
    }
#pragma unroll
    for (int j = 0; j < GPW; ++j) {
      float2 y[4];
      split::mma_group(F, X[j], y, lane);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int r = i < 2 ? g : g + 8, c = 2 * q + (i & 1);
        const int bo = obfly(j, c), kbo = bo & 15;
        const int pos = (bo - kbo) * 16 + kbo + r * 16;
        const Ctx& co = (i & 1) ? c1 : c0;
        if constexpr (KIND == K_R2C) co.put_r2c(S, pos, y[i]);
        else co.gstore(pos, y[i]);
      }
    }
    if constexpr (KIND == K_R2C) {
      __syncthreads();
      cs.store_r2c_pairs(S);
    }
  } else {
#pragma unroll
    for (int j = 0; j < GPW; ++j) {
      float2 y[4];
      split::mma_group(F, X[j], y, lane);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int r = i < 2 ? g : g + 8, c = 2 * q + (i & 1);
        const int bo = obfly(j, c), kbo = bo & 15;
        S[cm.sidx_at(oline(c), (bo - kbo) * 16 + kbo + r * 16)] = y[i];
      }
    }
    __syncthreads();

    // ---- stage 3: radix R = N / 256, NS = 256, CUDA cores ---------------------
    constexpr int R = N / 256, NBR = N / R;  // NBR = 256 butterflies a line
    constexpr int IPT = NBR / TPL;           // butterflies a thread
    float2 V[IPT][R];
#pragma unroll
    for (int j = 0; j < IPT; ++j) {
      const int b = st + j * TPL;  // b < NS: twiddle exponent k = b, outputs b + r NS
#pragma unroll
      for (int r = 0; r < R; ++r) V[j][r] = S[cs.sidx(b + r * NBR)];
#pragma unroll
      for (int r = 1; r < R; ++r) V[j][r] = cmul(V[j][r], cs.twiddle(255 + (r - 1) * 256 + b));
      dftp<R>(V[j]);
    }
    if constexpr (KIND == K_R2C) {
      __syncthreads();
#pragma unroll
      for (int j = 0; j < IPT; ++j)
#pragma unroll
        for (int r = 0; r < R; ++r) cs.put_r2c(S, st + j * TPL + r * 256, V[j][r]);
      __syncthreads();
      cs.store_r2c_pairs(S);
    } else {
#pragma unroll
      for (int j = 0; j < IPT; ++j)
#pragma unroll
        for (int r = 0; r < R; ++r) cs.gstore(st + j * TPL + r * 256, V[j][r]);
    }
  }
}

template <int KIND, bool CONTIG, int N>
cudaError_t launch_n(const PassArgs& a, cudaStream_t stream) {
  constexpr int L = CONTIG ? 4 : 8;
  if (a.L != L) return cudaErrorInvalidValue;
  const size_t smem = (size_t)fast_smem_entries(N, L) * sizeof(float2);
  auto kern = split_pass_kernel<KIND, CONTIG, N>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const dim3 grid((unsigned)((a.nlines + L - 1) / L), CONTIG ? 1u : (unsigned)a.nv);
  kern<<<grid, kThreads, smem, stream>>>(a);
  add_launches(1);
  return cudaGetLastError();
}

template <int KIND, bool CONTIG>
cudaError_t launch_k(const PassArgs& a, cudaStream_t s) {
  switch (a.n) {
    case 256: return launch_n<KIND, CONTIG, 256>(a, s);
    case 512: return launch_n<KIND, CONTIG, 512>(a, s);
    case 1024: return launch_n<KIND, CONTIG, 1024>(a, s);
    default: return cudaErrorNotSupported;
  }
}

}  // namespace

bool split_length(int n) { return n == 256 || n == 512 || n == 1024; }

int split_lines_per_cta(int n, bool contiguous) {
  (void)n;
  return contiguous ? 4 : 8;
}

cudaError_t launch_split_f32(int kind, bool contiguous, const PassArgs& a, cudaStream_t s) {
  if (kind == K_C2C) return contiguous ? launch_k<K_C2C, true>(a, s) : launch_k<K_C2C, false>(a, s);
  if (kind == K_R2C) return contiguous ? launch_k<K_R2C, true>(a, s) : launch_k<K_R2C, false>(a, s);
  return contiguous ? launch_k<K_C2R, true>(a, s) : launch_k<K_C2R, false>(a, s);
}

}  // namespace gbfft
