// Dense (non-diagonal) operator path with a per-instance controller: ETD35, ETD34 or IF34
// for a batch of instances sharing one n x n lin_op = S diag(eig) S^-1 (n <= 128, real
// spectrum), every instance with its own step size under the reference's accept/reject rule.
//
// The stepping follows the reference's diagonalized strategy (rkstiff/etd35.py:348-495,
// rkstiff/etd34.py:274-304, rkstiff/if34.py:164-196): the state is kept in the eigenbasis,
// v = S^-1 u; the stage combinations are elementwise with the diagonal coefficients of
// h_i eig (h_i the instance's step size, rebuilt when it changes); each nonlinear
// evaluation is S^-1 N(S k).  The two basis changes of a stage are 3xTF32 tcgen05 GEMMs
// (M = 128 vector rows, N = 64 instances per CTA, K = 128): the coefficient operand (S or
// S^-1, TF32 hi/lo) streams through a TMA ring, the stage operand is written by the previous
// epilogue straight into shared memory in the 128-byte swizzled K-major tile layout.  One
// persistent CTA per 64 instances loops over attempts:
//
//   ETD35, per attempt (13 GEMMs; 12 with the eigenbasis error vector):
//     k2 .. k6 (elementwise, eigenbasis) -> S k -> N (physical) -> S^-1 N -> N2 .. N6
//     unew, err (elementwise) -> S err (physical error vector, etd35.py:719) ->
//     S unew -> masked norms and s per instance (solveras.py:412-455) -> the reference's
//     accept/reject rule per instance (solveras.py:457-554) -> S^-1 N(S unew) = N1 of the
//     accepted state (ETD35 re-evaluates N(u) after an accepted step, etd35.py:310-318)
//   ETD34 / IF34, per attempt (9 GEMMs; 8 with the eigenbasis error vector):
//     k2 .. k4 -> N2 .. N4, unew -> S unew -> S^-1 N(S unew) = N5 -> err = c (N4 - N5) ->
//     S err -> error test and rule; N1 = N5 of an accepted attempt (first same as last)
//
// Warps 0-7 are the epilogues (thread = vector row, 32 instances each), warp 8 issues the
// MMAs, warp 9 the TMA loads.  Every wait is bounded by %globaltimer and reports through
// the CTA's instance records.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>
#include <type_traits>

#include "rk_evolve.cuh"
#include "rk_launch.h"
#include "rk_tc.cuh"

namespace rk {
namespace dense_eig {

constexpr int DM = RK_DENSE_NMAX;  // vector length (padded) = MMA M = K of a basis change
constexpr int NT = RK_DENSE_TILE;  // instances per CTA = MMA N
constexpr int KC = 32;             // K elements per chunk (128 bytes of FP32)
constexpr int NCH = DM / KC;       // chunks per GEMM
constexpr int NS = 4;              // ring slots (coefficient operand only)
constexpr int A_TILE = DM * KC * 4;
constexpr int B_TILE = NT * KC * 4;
constexpr int SLOT_BYTES = 2 * A_TILE;      // S or S^-1 chunk, hi and lo
constexpr int DEP_BYTES = 2 * NCH * B_TILE;  // stage operand: NCH hi tiles, then NCH lo tiles
constexpr int RED_BYTES = 3 * 4 * NT * 4;    // per-warp partial max, sum u^2, sum err^2
// the FP32 Taylor-series table of the method (rk_coef_series.cuh), copied to shared memory
constexpr int SER_FLOATS = sizeof(k_ser_etd35) / sizeof(float) > sizeof(k_ser_etd34) / sizeof(float)
                               ? (int)(sizeof(k_ser_etd35) / sizeof(float)) : (int)(sizeof(k_ser_etd34) / sizeof(float));
constexpr int SER_BYTES = (SER_FLOATS * 4 + 127) & ~127;
constexpr int SMEM = 1024 + NS * SLOT_BYTES + DEP_BYTES + RED_BYTES + 2048 + SER_BYTES;
// warps 0-7: epilogues (two per tensor-memory lane quarter, one per column half), warp 8:
// MMA issue, warp 9: TMA loads
constexpr int EPI_WARPS = 8, EPI_THREADS = 32 * EPI_WARPS;
constexpr int THREADS = EPI_THREADS + 64;
constexpr int MMA_TID = EPI_THREADS, PRODUCER_TID = EPI_THREADS + 32;
// tensor memory: the accumulator and the stage vectors of the attempt, NT columns each
enum { T_ACC, T_V, T_N1, T_N2, T_N3, T_N4, T_N5, T_UN, T_SLOTS };
constexpr int TMEM_COLS = T_SLOTS * NT;  // 512: the whole tensor memory of the SM
constexpr uint64_t WAIT_NS = 200000000ull;  // a wait gives up after 200 ms
enum { M_S = 0, M_SI = 1 };                 // coefficient operands
// per-instance vectors in global memory, instance-major with the row innermost: the
// eigenbasis state and its N1 between calls, the physical state
enum { V_V, V_N1, V_UP, NVEC };

struct Layout {
  int64_t bpad, a, v, c, eig, shift, total;
};
inline int64_t al1k(int64_t x) { return (x + 1023) & ~int64_t(1023); }
inline Layout layout(int64_t n_inst) {
  Layout L;
  L.bpad = (n_inst + NT - 1) / NT * NT;
  int64_t o = 0;
  L.a = o;
  o = al1k(o + (int64_t)2 * 2 * DM * DM * 4);
  L.v = o;
  o = al1k(o + (int64_t)NVEC * L.bpad * DM * 4);
  L.c = o;
  o = al1k(o + L.bpad * (int64_t)C35_N * DM * 4);
  L.eig = o;
  o = al1k(o + DM * 8);
  L.shift = o;
  o = al1k(o + DM * 4);
  L.total = o;
  return L;
}

struct Params {
  rk_inst_state* st;  // [n_inst]
  const float* A;     // [2 matrices][hi, lo][DM][DM]
  float* V;           // [NVEC][bpad][DM]
  float* C;           // [bpad][C35_N][DM]
  const double* eig;  // [DM]
  const float* shift; // [DM]
  float* u;           // caller's [n_inst][n] physical states
  int64_t n_inst, bpad;
  int n, err_eigen, first, max_attempts;
  rk_controller ctl;
  EtdCfg ec;
};

RK_DEV float* vec(const Params& p, int which, int64_t col) { return p.V + ((int64_t)which * p.bpad + col) * DM; }

// Allen-Cahn nonlinearity in the lifted form (rkstiff/models.py:242-244)
RK_DEV float nl_ac(float w, float x) {
  const float v = w + x;
  return x - v * v * v;
}

// FP32 coefficients of one real mode z = h lambda (layouts C35_*, C34_*, CIF_*): the stiff
// form below z = -STIFF_Z, the combinations' FP32 Taylor tables / stiff forms up to z = 80
// (series_coeffs_f32 reading the kernel's shared-memory copy `ser` of the table: the global
// table's lines missed the L1 left beside 198 KB of shared memory; 18.7 -> 17.6 ms for the
// 8192-IC ETD35 batch; IF34's exponentials in double-float), FP64 beyond.
template <int METHOD>
RK_DEV void mode_coeffs_f32(double z, double h, const EtdCfg& ec, float* out, const float* ser) {
  if (z < -(double)STIFF_Z) {
    stiff_coeffs_f32<METHOD>(z, h, out);
    return;
  }
  if constexpr (METHOD == RK_IF34) {
    // e^z and e^(z/2) (if34.py:109-112)
    if (z <= 80.0) {
      dd m;
      out[CIF_E] = dd_exp(dd_from_double(z), m).hi;
      out[CIF_E2] = dd_exp(dd_from_double(0.5 * z), m).hi;
    } else {
      out[CIF_E] = (float)exp(z);
      out[CIF_E2] = (float)exp(0.5 * z);
    }
  } else {
    constexpr int NP = METHOD == RK_ETD35 ? RK_PSI35_N : RK_PSI34_N;
    constexpr int NC = METHOD == RK_ETD35 ? C35_N : C34_N;
    if (z <= 80.0) {
      series_coeffs_f32<METHOD, true>(z, h, out, ser);
    } else {
      double E[4], P[NP], o[NC];
      fast_real_psi(METHOD, z, h, E, P);
      etd_from_psi_e<double>(METHOD, E, P, o);
#pragma unroll
      for (int c = 0; c < NC; ++c) out[c] = (float)o[c];
    }
  }
}
template <int METHOD> __host__ __device__ constexpr int num_coeffs() {
  return METHOD == RK_ETD35 ? (int)C35_N : METHOD == RK_ETD34 ? (int)C34_N : (int)CIF_N;
}

// Element (instance j, K row `row`) of the stage operand in shared memory: the tile of the
// row's 32-row chunk, instance j at 128 bytes, the 16-byte chunk (row % 32) / 4 XOR j % 8 --
// the layout a 128-byte-swizzled TMA load of a [NT][32] FP32 box produces.
RK_DEV int dep_index(int row, int j) {
  const int q = row >> 5, l = row & 31;
  return q * (B_TILE / 4) + j * 32 + ((((l >> 2) ^ (j & 7)) << 2) | (l & 3));
}
RK_DEV void dep_put(float* dep, int row, int j, float v) {
  const float hi = tc::tf32_hi(v);
  const int f = dep_index(row, j);
  dep[f] = hi;
  dep[f + DEP_BYTES / 8] = v - hi;
}

// 32 accumulator columns [half*32, half*32+32) of this thread's lane (row), accumulator
// at tensor-memory column offset acc * NT
RK_DEV void load_acc_half(uint32_t tmem, int warp, int acc, int half, float* v) {
  __syncwarp();  // tcgen05.ld is warp-collective
  const uint32_t base = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(acc * NT + half * 32);
  tc::tmem_ld16(base, v);
  tc::tmem_ld16(base + 16u, v + 16);
  tc::tmem_ld_wait();
}

// Reduce-scatter over the 32 lanes of a warp: v[32] per lane in, the reduction of column
// `lane` out in v[0] (31 shuffles).
template <class Op>
RK_DEV void warp_reduce_scatter32(float* v, int lane, Op op) {
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const bool up = lane & 16;
    const float keep = up ? v[16 + k] : v[k], send = up ? v[k] : v[16 + k];
    v[k] = op(keep, __shfl_xor_sync(0xffffffffu, send, 16));
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const bool up = lane & 8;
    const float keep = up ? v[8 + k] : v[k], send = up ? v[k] : v[8 + k];
    v[k] = op(keep, __shfl_xor_sync(0xffffffffu, send, 8));
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const bool up = lane & 4;
    const float keep = up ? v[4 + k] : v[k], send = up ? v[k] : v[4 + k];
    v[k] = op(keep, __shfl_xor_sync(0xffffffffu, send, 4));
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const bool up = lane & 2;
    const float keep = up ? v[2 + k] : v[k], send = up ? v[k] : v[2 + k];
    v[k] = op(keep, __shfl_xor_sync(0xffffffffu, send, 2));
  }
  v[0] = op(lane & 1 ? v[1] : v[0], __shfl_xor_sync(0xffffffffu, lane & 1 ? v[0] : v[1], 1));
}

// ---------------------------------------------------------------------------------
// set-up: S and S^-1 as TF32 hi/lo pairs (rows and columns n..127 zero), eig, shift
// ---------------------------------------------------------------------------------
__global__ void setup_kernel(float* A, double* eig_p, float* shift_p, int n, const double* eig, const double* S,
                             const double* Si, const double* shift) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < (int64_t)DM * DM) {
    const int r = (int)(i / DM), c = (int)(i % DM);
    const bool in = r < n && c < n;
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      const double v = in ? (m == M_S ? S : Si)[r * n + c] : 0.0;
      const float hi = tc::tf32_hi((float)v);
      A[((int64_t)(m * 2 + 0) * DM + r) * DM + c] = hi;
      A[((int64_t)(m * 2 + 1) * DM + r) * DM + c] = (float)(v - (double)hi);
    }
  }
  if (i < DM) {
    eig_p[i] = i < n ? eig[i] : 0.0;
    shift_p[i] = i < n ? (float)shift[i] : 0.f;
  }
}

// Coefficient operand of GEMM q of an attempt of L GEMMs.  ETD35: the five stages
// alternate S (to physical space) and S^-1 (back), then S err (physical error vector only),
// S unew, S^-1 N(unew).  ETD34 / IF34: three stages and S unew -> S^-1 N(unew) alternate,
// then S err (physical error vector only).
template <int METHOD>
RK_DEV int attempt_matrix(int q, int L) {
  if constexpr (METHOD == RK_ETD35) {
    if (q < 10) return (q & 1) ? M_SI : M_S;
    return q == L - 1 ? M_SI : M_S;
  } else {
    return (q < 8 && (q & 1)) ? M_SI : M_S;
  }
}

// the reference's accept/reject rule (solveras.py:457-554, the evolve loop's end-time
// clamp, solveras.py:622-640) for one instance; returns 1 when the attempt is accepted
// ETD35 evaluates N five times per attempt and N(unew) after an accepted one; the FSAL
// methods (ETD34, IF34) four times per attempt, the last of them being N(unew).
RK_DEV int control_instance(rk_inst_state& s, double sv, const rk_controller& ctl, bool fsal) {
  const double h = s.h;
  s.attempts += 1;
  s.nl_evals += fsal ? 4 : 5;
  s.s_last = sv;
  if (isinf(sv) || isnan(sv) || sv < 1.0) {
    s.accept = 0;
    s.rejects += 1;
    s.h = reject_h(sv, h, ctl);
    s.reserved_i += 1;  // attempts since the last accepted step
    if (s.reserved_i > 50) s.status = RK_ST_MAX_LOOPS;
    else if (s.h < ctl.minh) s.status = RK_ST_MIN_STEP;
    return 0;
  }
  s.accept = 1;
  if (!fsal) s.nl_evals += 1;  // N(unew), the next attempt's N1
  const double t = s.t + h;
  s.t = t;
  s.steps += 1;
  s.reserved_i = 0;
  s.h_used = h;
  const double hs = accept_h(sv, h, ctl);
  s.h_suggest = hs;
  const double hn = (t + hs > s.tf) ? s.tf - t : hs;
  s.h = hn;
  if (!(t < s.tf)) s.status = RK_ST_DONE;
  else if (t + hn == t) s.status = RK_ST_MIN_STEP;
  return 1;
}

// ---------------------------------------------------------------------------------
// the persistent kernel: one CTA per NT instances, attempts until every instance of the
// CTA has finished or max_attempts attempts ran
// ---------------------------------------------------------------------------------
// Barrier phases: depr and accb complete once per GEMM (the stage operand of GEMM q is in
// shared memory / GEMM q's accumulator is complete), go once per decision (decision 0 at the
// start, decision a + 1 after attempt a's error test: continue or stop, in flags[0]).
template <int METHOD>
__global__ void __launch_bounds__(THREADS, 1) eig_kernel(const __grid_constant__ CUtensorMap tmA, Params p) {
  extern __shared__ unsigned char smem_raw[];
  // 1024-byte aligned by pointer arithmetic on the shared array (not through an integer),
  // so that the compiler knows every pointer below addresses shared memory
  unsigned char* sm = smem_raw + ((1024u - (uint32_t)(reinterpret_cast<uintptr_t>(smem_raw) & 1023u)) & 1023u);
  float* dep = reinterpret_cast<float*>(sm + NS * SLOT_BYTES);
  float* red = reinterpret_cast<float*>(sm + NS * SLOT_BYTES + DEP_BYTES);  // [3][4 warps][NT]
  unsigned char* ctl_area = sm + NS * SLOT_BYTES + DEP_BYTES + RED_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(ctl_area);
  uint64_t* empty = full + NS;
  uint64_t* accb = empty + NS;
  uint64_t* depr = accb + 1;
  uint64_t* go = depr + 1;
  uint64_t* xb = go + 1;  // exchanges among the epilogue threads (bounded, unlike bar.sync)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(xb + 1);
  volatile int* flags = reinterpret_cast<volatile int*>(tmem_slot + 1);  // [0] stop, [1] abort
  double* hsm = reinterpret_cast<double*>(ctl_area + 256);               // [NT] h of each instance
  int* need = reinterpret_cast<int*>(hsm + NT);                          // [NT] coefficients to rebuild
  int* acc_ok = need + NT;                                               // [NT] attempt accepted
  int* running = acc_ok + NT;                                            // [NT] instance running
  int* stiffq = running + NT;  // [NT] bit q: every row of chunk q of the instance is stiff at its h
  double* lamq = reinterpret_cast<double*>(stiffq + NT);                 // [4] largest eig of each chunk
  unsigned* needw = reinterpret_cast<unsigned*>(lamq + DM / 32);         // [2] need[] as a bit mask
  float* ser = reinterpret_cast<float*>(ctl_area + 2048);                 // series table copy

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t col0 = (int64_t)blockIdx.x * NT;
  // GEMMs per attempt (one fewer with the eigenbasis error vector)
  const int L = METHOD == RK_ETD35 ? (p.err_eigen ? 12 : 13) : (p.err_eigen ? 8 : 9);
  constexpr int NCF = num_coeffs<METHOD>();

  if (tid == 0) {
    for (int i = 0; i < NS; ++i) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    tc::mbar_init(accb, 1);
    tc::mbar_init(depr, EPI_THREADS);
    tc::mbar_init(go, EPI_THREADS);
    tc::mbar_init(xb, EPI_THREADS);
    flags[0] = 0;
    flags[1] = 0;
    for (int q = 0; q < DM / 32; ++q) {
      double m = p.eig[q * 32];
      for (int r = q * 32 + 1; r < q * 32 + 32; ++r) m = fmax(m, p.eig[r]);
      lamq[q] = m;
    }
    tc::fence_mbar_init();
    tc::prefetch_tmap(&tmA);
  }
  if constexpr (METHOD == RK_ETD35 || METHOD == RK_ETD34) {
    // the rebuilds' Taylor-series table, read by every non-stiff mode (published by the
    // __syncthreads below)
    constexpr int nf = (int)((METHOD == RK_ETD35 ? sizeof(k_ser_etd35) : sizeof(k_ser_etd34)) / sizeof(float));
    const float* src = METHOD == RK_ETD35 ? k_ser_etd35 : k_ser_etd34;
    for (int i = tid; i < nf; i += THREADS) ser[i] = src[i];
  }
  __syncwarp();
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, TMEM_COLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (tid == PRODUCER_TID) {
    // the coefficient operand of every GEMM, chunk by chunk, into the ring; the loads of an
    // attempt are issued once the decision to run it is known
    int g = 0;
    auto load_gemm = [&](int m) -> bool {
      for (int c = 0; c < NCH; ++c, ++g) {
        const int slot = g % NS;
        if (g >= NS && !tc::mbar_wait(&empty[slot], (uint32_t)((g / NS) - 1) & 1u, WAIT_NS)) return false;
        unsigned char* base = sm + slot * SLOT_BYTES;
        tc::mbar_arrive_expect_tx(&full[slot], (uint32_t)SLOT_BYTES);
        tc::tma_load_2d(base, &tmA, &full[slot], c * KC, (m * 2 + 0) * DM);
        tc::tma_load_2d(base + A_TILE, &tmA, &full[slot], c * KC, (m * 2 + 1) * DM);
      }
      return true;
    };
    bool ok = tc::mbar_wait(go, 0u, WAIT_NS);
    if (ok && !flags[0]) {
      if (p.first) ok = load_gemm(M_SI) && load_gemm(M_SI);
      for (int d = 1; ok; ++d) {
        for (int q = 0; q < L && ok; ++q) ok = load_gemm(attempt_matrix<METHOD>(q, L));
        if (ok) ok = tc::mbar_wait(go, (uint32_t)d & 1u, WAIT_NS);
        if (flags[0] || flags[1]) break;
      }
    }
    if (!ok) flags[1] = 1;
    // copies still in flight land before the CTA exits: the last NS chunks' full barriers
    for (int k = g - NS > 0 ? g - NS : 0; k < g; ++k) tc::mbar_wait(&full[k % NS], (uint32_t)(k / NS) & 1u, WAIT_NS);
  } else if (tid == MMA_TID) {
    constexpr uint32_t idesc = tc::idesc_tf32(DM, NT);
    const uint32_t dep_s = tc::smem_u32(dep);
    int g = 0, q = 0;
    auto run_gemm = [&]() -> bool {
      if (!tc::mbar_wait(depr, (uint32_t)q & 1u, WAIT_NS)) return false;
      tc::tc_fence_after();
      for (int c = 0; c < NCH; ++c, ++g) {
        const int slot = g % NS;
        if (!tc::mbar_wait(&full[slot], (uint32_t)(g / NS) & 1u, WAIT_NS)) return false;
        tc::tc_fence_after();
        const uint32_t sa = tc::smem_u32(sm + slot * SLOT_BYTES);
        const uint64_t ahi = tc::sdesc_kmajor_sw128(sa), alo = tc::sdesc_kmajor_sw128(sa + A_TILE);
        const uint64_t bhi = tc::sdesc_kmajor_sw128(dep_s + (uint32_t)(c * B_TILE));
        const uint64_t blo = tc::sdesc_kmajor_sw128(dep_s + (uint32_t)(DEP_BYTES / 2 + c * B_TILE));
#pragma unroll
        for (int kk = 0; kk < KC / 8; ++kk) {
          const uint64_t o = (uint64_t)((kk * 32) >> 4);  // 8 TF32 = 32 bytes along K
          tc::mma_tf32(tmem, alo + o, bhi + o, idesc, (c == 0 && kk == 0) ? 0u : 1u);
          tc::mma_tf32(tmem, ahi + o, blo + o, idesc, 1u);
          tc::mma_tf32(tmem, ahi + o, bhi + o, idesc, 1u);
        }
        tc::mma_commit(&empty[slot]);
      }
      tc::mma_commit(accb);
      ++q;
      return true;
    };
    bool ok = tc::mbar_wait(go, 0u, WAIT_NS);
    if (ok && !flags[0]) {
      if (p.first) ok = run_gemm() && run_gemm();
      for (int d = 1; ok; ++d) {
        for (int i = 0; i < L && ok; ++i) ok = run_gemm();
        if (ok) ok = tc::mbar_wait(go, (uint32_t)d & 1u, WAIT_NS);
        if (flags[0] || flags[1]) break;
      }
    }
    if (!ok) flags[1] = 1;
  } else if (warp < EPI_WARPS) {
    // epilogues: thread = vector row `row` (tensor-memory lane quarter warp % 4) for the 32
    // instances of column half `ch` (warps 0-3: instances 0-31, warps 4-7: 32-63); threads
    // 0..NT-1 also run the controller of instance col0 + tid.  The stage vectors of the
    // attempt live in tensor memory (slots T_V .. T_UN beside the accumulator); only the
    // coefficients and the physical state are read or written in global memory.
    const int row = tid & (DM - 1), ch = tid >> 7, quarter = warp & 3;
    const int j0 = ch * 32;
    const float xr = p.shift[row];
    const bool own = tid < NT && col0 + tid < p.n_inst;
    rk_inst_state so{};
    if (own) so = p.st[col0 + tid];
    bool ok = true;
    int q = 0;  // GEMMs completed (accb phases)
    float acc[32], e2[32], u2[32];
    auto publish = [&]() {
      tc::fence_proxy_async_shared();
      tc::tc_fence_before();
      tc::mbar_arrive(depr);
    };
    auto wait_acc = [&]() -> bool {
      const bool w = tc::mbar_wait(accb, (uint32_t)q & 1u, WAIT_NS);
      ++q;
      tc::tc_fence_after();
      if (!w) flags[1] = 1;
      return w && !flags[1];
    };
    auto load_acc = [&]() { load_acc_half(tmem, quarter, T_ACC, ch, acc); };
    // tensor-memory columns [slot*NT + ch*32 + sub*16, +16) of this warp's lane quarter
    auto taddr = [&](int slot, int sub) {
      return tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(slot * NT + ch * 32 + sub * 16);
    };
    auto tld = [&](int slot, int sub, float* v) { tc::tmem_ld16(taddr(slot, sub), v); };
    auto tst = [&](int slot, int sub, const float* v) { tc::tmem_st16(taddr(slot, sub), v); };
    // coefficient loads through the global state space (ld.global.ca), so that the compiler
    // may move them past the shared-memory stores of the stage operand; each thread reads
    // the entries of its own row and instances, which it wrote itself
    auto cf = [&](int j, int c) { return __ldca(p.C + ((col0 + j) * C35_N + c) * DM + row); };
    auto V = [&](int which, int j) -> float& { return vec(p, which, col0 + j)[row]; };
    // all epilogue threads meet; a thread that gave up on an earlier wait never arrives, so
    // the others time out here instead of waiting forever
    int xphase = 0;
    auto sync_epi = [&]() -> bool {
      tc::mbar_arrive(xb);
      const bool w = tc::mbar_wait(xb, (uint32_t)xphase & 1u, WAIT_NS);
      ++xphase;
      if (!w) flags[1] = 1;
      return w;
    };
    auto publish_state = [&]() {
      if (tid < NT) {
        running[tid] = own && so.status == RK_ST_RUNNING;
        hsm[tid] = own ? so.h : 0.0;
        const bool nd = own && so.status == RK_ST_RUNNING && so.h != so.h_coeff;  // exact, as etd35.py:851
        need[tid] = nd;
        const unsigned b = __ballot_sync(0xffffffffu, nd);  // warps 0 and 1, all lanes
        if (lane == 0) needw[warp] = b;
        int m = 0;
        for (int q = 0; q < DM / 32; ++q) m |= (hsm[tid] * lamq[q] < -(double)STIFF_Z) ? (1 << q) : 0;
        stiffq[tid] = m;
      }
    };
    // decision 0
    publish_state();
    tc::named_sync(1, EPI_THREADS);
    if (tid == 0) {
      int any = 0;
      for (int j = 0; j < NT; ++j) any |= running[j];
      flags[0] = (!any || p.max_attempts < 1) ? 1 : 0;
    }
    tc::named_sync(1, EPI_THREADS);
    const bool stop0 = flags[0] != 0;
    tc::mbar_arrive(go);
    bool have_state = !p.first;  // v, N1 in global memory and V_UP valid
    if (!stop0 && p.first) {
      // v = S^-1 u and N1 = S^-1 N(u) from the caller's physical states
#pragma unroll 8
      for (int jj = 0; jj < 32; ++jj) {
        const int64_t col = col0 + j0 + jj;
        const float uv = (col < p.n_inst && row < p.n) ? p.u[col * p.n + row] : 0.f;
        V(V_UP, j0 + jj) = uv;
        dep_put(dep, row, j0 + jj, uv);
      }
      have_state = true;
      publish();
      ok = wait_acc();
      if (ok) {
        load_acc();
        tst(T_V, 0, acc);
        tst(T_V, 1, acc + 16);
#pragma unroll 8
        for (int jj = 0; jj < 32; ++jj) dep_put(dep, row, j0 + jj, nl_ac(__ldca(vec(p, V_UP, col0 + j0 + jj) + row), xr));
        tc::tmem_st_wait();
        publish();
        ok = wait_acc();
      }
      if (ok) {
        load_acc();
        tst(T_N1, 0, acc);
        tst(T_N1, 1, acc + 16);
        tc::tmem_st_wait();
        if (own && so.status == RK_ST_RUNNING) so.nl_evals += 1;  // the first N(u)
      }
    } else if (!stop0) {
      // v and N1 of the current state from the previous call
#pragma unroll
      for (int sub = 0; sub < 2; ++sub) {
        float a[16], b[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          a[k] = V(V_V, j0 + sub * 16 + k);
          b[k] = V(V_N1, j0 + sub * 16 + k);
        }
        tst(T_V, sub, a);
        tst(T_N1, sub, b);
      }
      tc::tmem_st_wait();
    }
    // The error test of an attempt and the decision on the next (solveras.py:412-455 and
    // 457-554 per instance): u2 holds |S unew|^2 per instance (NaN as +inf, which leaves
    // every mask false and s NaN, as in the reference), acc the physical unew, e2 err^2.
    // Max |u|^2 over the rows, then the sums of u^2 and err^2 over the rows with u^2 >
    // cutoff^2 max |u|^2.  Rows: the 32 lanes of a warp (reduce-scatter: lane l ends with
    // instance j0 + l) and the four lane quarters (shared memory).
    auto error_test = [&](int a, bool& stop) -> bool {
      warp_reduce_scatter32(u2, lane, [](float x, float y) { return fmaxf(x, y); });
      red[(0 * 4 + quarter) * NT + j0 + lane] = u2[0];
      if (!sync_epi()) return false;
      const float cut2 = (float)(p.ctl.adapt_cutoff * p.ctl.adapt_cutoff);
#pragma unroll
      for (int jj = 0; jj < 32; ++jj) {
        const int j = j0 + jj;
        const float mx = fmaxf(fmaxf(red[j], red[NT + j]), fmaxf(red[2 * NT + j], red[3 * NT + j]));
        const float up = acc[jj], a2 = up * up;
        const bool m = a2 > cut2 * mx;
        u2[jj] = m ? a2 : 0.f;
        e2[jj] = m ? e2[jj] : 0.f;
      }
      warp_reduce_scatter32(u2, lane, [](float x, float y) { return x + y; });
      warp_reduce_scatter32(e2, lane, [](float x, float y) { return x + y; });
      red[(1 * 4 + quarter) * NT + j0 + lane] = u2[0];
      red[(2 * 4 + quarter) * NT + j0 + lane] = e2[0];
      if (!sync_epi()) return false;
      if (tid < NT) {
        acc_ok[tid] = 0;
        if (own && so.status == RK_ST_RUNNING) {
          double su = 0.0, se = 0.0;
          for (int w = 0; w < 4; ++w) {
            su += (double)red[(1 * 4 + w) * NT + tid];
            se += (double)red[(2 * 4 + w) * NT + tid];
          }
          // s = safety (eps |u| / |err|)^(1/q), q = 4, as ratio^(1/8) of ratio = eps^2 su / se.
          // An error vector that is exactly zero in FP32 while |u| > 0 (IF34's h (N4 - N5) / 6
          // on a short last step) lies below FP32 resolution: the largest growth, MAX_S = 4,
          // instead of the rejection x/0 = inf would give.
          const double ratio = (p.ctl.epsilon * p.ctl.epsilon * su) / se;
          const double sv = (se == 0.0 && su > 0.0 && !isinf(su)) ? 4.0
                            : (ratio != ratio || isinf(ratio)) ? p.ctl.safety_f * ratio
                                                               : p.ctl.safety_f * pow(ratio, 0.125);
          acc_ok[tid] = control_instance(so, sv, p.ctl, METHOD != RK_ETD35);
        }
      }
      publish_state();
      if (!sync_epi()) return false;
      if (tid == 0) {
        int any = 0;
        for (int j = 0; j < NT; ++j) any |= running[j];
        flags[0] = (!any || a + 1 >= p.max_attempts) ? 1 : 0;
      }
      if (!sync_epi()) return false;
      stop = flags[0] != 0;
      tc::mbar_arrive(go);
      return true;
    };
    for (int a = 0; ok && !stop0; ++a) {
      // Coefficients of the instances whose h changed, in units of (instance j, 32-row chunk
      // q) dealt round-robin to the eight epilogue warps: first the units with a row that is
      // not stiff (double-float psi functions), then the all-stiff ones (FP32), so that every
      // warp gets a like share of the slow work.  Lane l computes row 32 q + l; each value
      // depends only on its own h lambda, whichever warp computes it.
      const unsigned long long nmask = (unsigned long long)needw[0] | ((unsigned long long)needw[1] << 32);
      if (nmask) {
        int u = 0;
        for (int pass = 0; pass < 2; ++pass) {
          for (unsigned long long mk = nmask; mk; mk &= mk - 1) {
            const int j = __ffsll((long long)mk) - 1;
            const int sq = stiffq[j];
            for (int q = 0; q < DM / 32; ++q) {
              if (((sq >> q) & 1) != pass) continue;
              if ((u++ & (EPI_WARPS - 1)) != warp) continue;
              const int r = q * 32 + lane;
              float c[NCF];
              const double h = hsm[j];
              mode_coeffs_f32<METHOD>(h * p.eig[r], h, p.ec, c, ser);
              float* cp = p.C + ((col0 + j) * C35_N) * DM + r;
#pragma unroll
              for (int k = 0; k < NCF; ++k) cp[k * DM] = c[k];
            }
          }
        }
      }
      if (own && need[tid]) {
        so.h_coeff = so.h;
        so.coeff_updates += 1;
      }
      if (nmask) {
        // the coefficients written by other warps, visible before the stages read them
        __threadfence_block();
        if (!(ok = sync_epi())) break;
      }
      bool stop = false;
      if constexpr (METHOD == RK_ETD35) {
        // k2 = E14 v + a21 N1 (etd35.py:320)
#pragma unroll
        for (int sub = 0; sub < 2; ++sub) {
          float v[16], n1[16];
          tld(T_V, sub, v);
          tld(T_N1, sub, n1);
          tc::tmem_ld_wait();
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const int j = j0 + sub * 16 + k;
            dep_put(dep, row, j, cf(j, C35_E14) * v[k] + cf(j, C35_A21) * n1[k]);
          }
        }
        publish();
        // stages 2..6: S k -> N in physical space -> S^-1 N = N_st; the next combination.  One
        // instantiation per stage, so that each keeps only the vectors it reads live.
        auto stage = [&](auto stc) -> bool {
          constexpr int st = decltype(stc)::value;
          if (!wait_acc()) return false;
          load_acc();
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) dep_put(dep, row, j0 + jj, nl_ac(acc[jj], xr));
          publish();
          if (!wait_acc()) return false;
#pragma unroll
          for (int sub = 0; sub < 2; ++sub) {
            float nk[16], v[16], n1[16], x1[16], x2[16], x3[16];
            tld(T_ACC, sub, nk);
            tld(T_V, sub, v);
            tld(T_N1, sub, n1);
            if constexpr (st == 4) {
              tld(T_N2, sub, x1);
              tld(T_N3, sub, x2);
            } else if constexpr (st == 5) {
              tld(T_N2, sub, x1);
              tld(T_N3, sub, x2);
              tld(T_N4, sub, x3);
            } else if constexpr (st == 6) {
              tld(T_N3, sub, x1);
              tld(T_N4, sub, x2);
              tld(T_N5, sub, x3);
            }
            tc::tmem_ld_wait();
#pragma unroll
            for (int k = 0; k < 16; ++k) {
              const int j = j0 + sub * 16 + k;
              // etd35.py:322-345
              if constexpr (st == 2) {
                dep_put(dep, row, j, (cf(j, C35_E14) * v[k] + cf(j, C35_A31) * n1[k]) + cf(j, C35_A32) * nk[k]);
              } else if constexpr (st == 3) {
                dep_put(dep, row, j, (cf(j, C35_E12) * v[k] + cf(j, C35_A41) * n1[k]) + cf(j, C35_A43) * nk[k]);
              } else if constexpr (st == 4) {
                dep_put(dep, row, j,
                        ((cf(j, C35_E34) * v[k] + cf(j, C35_A51) * n1[k]) + cf(j, C35_A52) * (x1[k] - x2[k])) +
                            cf(j, C35_A54) * nk[k]);
              } else if constexpr (st == 5) {
                const float t = x1[k] - (3.f * x3[k]) * 0.5f;
                dep_put(dep, row, j,
                        (((cf(j, C35_E) * v[k] + cf(j, C35_A61) * n1[k]) + cf(j, C35_A62) * t) + cf(j, C35_A63) * x2[k]) +
                            cf(j, C35_A65) * nk[k]);
              } else {
                const float un = ((((cf(j, C35_E) * v[k] + cf(j, C35_A71) * n1[k]) + cf(j, C35_A73) * x1[k]) +
                                   cf(j, C35_A74) * x2[k]) + cf(j, C35_A75) * x3[k]) + cf(j, C35_A76) * nk[k];
                const float er =
                    cf(j, C35_A75) * ((((-n1[k] + 4.f * x1[k]) - 6.f * x2[k]) + 4.f * x3[k]) - nk[k]);
                nk[k] = un;  // stored as unew below
                if (p.err_eigen) e2[sub * 16 + k] = er * er;
                else dep_put(dep, row, j, er);
              }
            }
            tst(st < 6 ? T_N2 + st - 2 : T_UN, sub, nk);
          }
          tc::tmem_st_wait();
          if constexpr (st < 6) publish();
          return true;
        };
        ok = stage(std::integral_constant<int, 2>{}) && stage(std::integral_constant<int, 3>{}) &&
             stage(std::integral_constant<int, 4>{}) && stage(std::integral_constant<int, 5>{}) &&
             stage(std::integral_constant<int, 6>{});
        if (!ok) break;
        if (!p.err_eigen) {
          // S err: the error vector in physical space (etd35.py:719)
          publish();
          if (!(ok = wait_acc())) break;
          load_acc();
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) e2[jj] = acc[jj] * acc[jj];
        }
#pragma unroll
        for (int sub = 0; sub < 2; ++sub) {
          float un[16];
          tld(T_UN, sub, un);
          tc::tmem_ld_wait();
#pragma unroll
          for (int k = 0; k < 16; ++k) dep_put(dep, row, j0 + sub * 16 + k, un[k]);
        }
        publish();
        if (!(ok = wait_acc())) break;
        // S unew: the physical new state; N(S unew) for the next attempt's N1
        load_acc();
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) {
          const float up = acc[jj];
          const float a2 = up * up;
          u2[jj] = a2 != a2 ? INFINITY : a2;
          dep_put(dep, row, j0 + jj, nl_ac(up, xr));
        }
        publish();
        if (!(ok = error_test(a, stop))) break;
        // the physical new state is in acc until the next load; keep it in u2 for the update
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) u2[jj] = acc[jj];
        if (!(ok = wait_acc())) break;
        // accepted instances take the new state and N1 = S^-1 N(S unew)
#pragma unroll
        for (int sub = 0; sub < 2; ++sub) {
          float n1n[16], n1[16], v[16], un[16];
          tld(T_ACC, sub, n1n);
          tld(T_N1, sub, n1);
          tld(T_V, sub, v);
          tld(T_UN, sub, un);
          tc::tmem_ld_wait();
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const int j = j0 + sub * 16 + k;
            if (acc_ok[j]) {
              n1[k] = n1n[k];
              v[k] = un[k];
              V(V_UP, j) = u2[sub * 16 + k];
            }
          }
          tst(T_N1, sub, n1);
          tst(T_V, sub, v);
        }
        tc::tmem_st_wait();
      } else {
        // k2 (etd34.py:293, if34.py:185)
#pragma unroll
        for (int sub = 0; sub < 2; ++sub) {
          float v[16], n1[16];
          tld(T_V, sub, v);
          tld(T_N1, sub, n1);
          tc::tmem_ld_wait();
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const int j = j0 + sub * 16 + k;
            if constexpr (METHOD == RK_ETD34) {
              dep_put(dep, row, j, cf(j, C34_E2) * v[k] + cf(j, C34_A21) * n1[k]);
            } else {
              const float e2c = cf(j, CIF_E2);
              dep_put(dep, row, j, e2c * v[k] + (0.5f * (float)hsm[j]) * (e2c * n1[k]));
            }
          }
        }
        publish();
        // stages 2..4: S k -> N in physical space -> S^-1 N = N_st; the next combination, the
        // last of them unew (written as the operand of S unew).  One instantiation per stage.
        auto stage = [&](auto stc) -> bool {
          constexpr int st = decltype(stc)::value;
          if (!wait_acc()) return false;
          load_acc();
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) dep_put(dep, row, j0 + jj, nl_ac(acc[jj], xr));
          publish();
          if (!wait_acc()) return false;
#pragma unroll
          for (int sub = 0; sub < 2; ++sub) {
            float nk[16], v[16], n1[16], x1[16], x2[16];
            tld(T_ACC, sub, nk);
            tld(T_V, sub, v);
            if constexpr (METHOD == RK_ETD34 || st == 4) tld(T_N1, sub, n1);
            if constexpr (st == 4) {
              tld(T_N2, sub, x1);
              tld(T_N3, sub, x2);
            }
            tc::tmem_ld_wait();
#pragma unroll
            for (int k = 0; k < 16; ++k) {
              const int j = j0 + sub * 16 + k;
              float kv;
              if constexpr (METHOD == RK_ETD34) {
                // etd34.py:295-301
                if constexpr (st == 2) {
                  kv = (cf(j, C34_E2) * v[k] + cf(j, C34_A31) * n1[k]) + cf(j, C34_A32) * nk[k];
                } else if constexpr (st == 3) {
                  kv = (cf(j, C34_E) * v[k] + cf(j, C34_A41) * n1[k]) + cf(j, C34_A43) * nk[k];
                } else {
                  kv = ((cf(j, C34_E) * v[k] + cf(j, C34_A51) * n1[k]) + cf(j, C34_A52) * (x1[k] + x2[k])) +
                       cf(j, C34_A54) * nk[k];
                }
              } else {
                // if34.py:186-193
                const float h = (float)hsm[j];
                if constexpr (st == 2) {
                  kv = cf(j, CIF_E2) * v[k] + (0.5f * h) * nk[k];
                } else if constexpr (st == 3) {
                  kv = cf(j, CIF_E) * v[k] + h * (cf(j, CIF_E2) * nk[k]);
                } else {
                  const float e = cf(j, CIF_E), e2c = cf(j, CIF_E2);
                  kv = e * v[k] + h * ((((e * n1[k]) * (1.f / 6.f) + (e2c * x1[k]) * (1.f / 3.f)) +
                                        (e2c * x2[k]) * (1.f / 3.f)) + nk[k] * (1.f / 6.f));
                }
              }
              dep_put(dep, row, j, kv);
              if constexpr (st == 4) v[k] = kv;
            }
            tst(T_N2 + st - 2, sub, nk);
            if constexpr (st == 4) tst(T_UN, sub, v);
          }
          tc::tmem_st_wait();
          publish();
          return true;
        };
        ok = stage(std::integral_constant<int, 2>{}) && stage(std::integral_constant<int, 3>{}) &&
             stage(std::integral_constant<int, 4>{});
        if (!ok) break;
        // S unew: the physical new state (kept in the free slot T_N2 for the update) ->
        // N(S unew) -> S^-1 N = N5, the next attempt's N1 when accepted
        if (!(ok = wait_acc())) break;
        load_acc();
        tst(T_N2, 0, acc);
        tst(T_N2, 1, acc + 16);
#pragma unroll
        for (int jj = 0; jj < 32; ++jj) {
          const float up = acc[jj], a2 = up * up;
          u2[jj] = a2 != a2 ? INFINITY : a2;
          dep_put(dep, row, j0 + jj, nl_ac(up, xr));
        }
        tc::tmem_st_wait();
        publish();
        if (!(ok = wait_acc())) break;
        // err = a54 (N4 - N5) (etd34.py:303) or h (N4 - N5) / 6 (if34.py:195)
#pragma unroll
        for (int sub = 0; sub < 2; ++sub) {
          float n5[16], n4[16];
          tld(T_ACC, sub, n5);
          tld(T_N4, sub, n4);
          tc::tmem_ld_wait();
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const int j = j0 + sub * 16 + k;
            const float c = METHOD == RK_ETD34 ? cf(j, C34_A54) : (float)hsm[j] * (1.f / 6.f);
            const float er = c * (n4[k] - n5[k]);
            if (p.err_eigen) e2[sub * 16 + k] = er * er;
            else dep_put(dep, row, j, er);
          }
          tst(T_N5, sub, n5);
        }
        tc::tmem_st_wait();
        if (!p.err_eigen) {
          // S err: the error vector in physical space (the non-diagonal form's err)
          publish();
          if (!(ok = wait_acc())) break;
          load_acc();
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) e2[jj] = acc[jj] * acc[jj];
        }
        // the physical new state back into acc for the error test
        tld(T_N2, 0, acc);
        tld(T_N2, 1, acc + 16);
        tc::tmem_ld_wait();
        if (!(ok = error_test(a, stop))) break;
        // accepted instances take the new state and N1 = N5 (FSAL)
#pragma unroll
        for (int sub = 0; sub < 2; ++sub) {
          float n5[16], n1[16], v[16], un[16];
          tld(T_N5, sub, n5);
          tld(T_N1, sub, n1);
          tld(T_V, sub, v);
          tld(T_UN, sub, un);
          tc::tmem_ld_wait();
#pragma unroll
          for (int k = 0; k < 16; ++k) {
            const int j = j0 + sub * 16 + k;
            if (acc_ok[j]) {
              n1[k] = n5[k];
              v[k] = un[k];
              V(V_UP, j) = acc[sub * 16 + k];
            }
          }
          tst(T_N1, sub, n1);
          tst(T_V, sub, v);
        }
        tc::tmem_st_wait();
      }
      if (stop) break;
    }
    if (!ok) flags[1] = 1;
    if (own) {
      if (!ok) so.status = RK_ST_WAIT_TIMEOUT;
      p.st[col0 + tid] = so;
    }
    if (have_state && !stop0) {
      // v and N1 of the current state for the next call
#pragma unroll
      for (int sub = 0; sub < 2; ++sub) {
        float v[16], n1[16];
        tld(T_V, sub, v);
        tld(T_N1, sub, n1);
        tc::tmem_ld_wait();
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          V(V_V, j0 + sub * 16 + k) = v[k];
          V(V_N1, j0 + sub * 16 + k) = n1[k];
        }
      }
    }
    if (have_state && row < p.n) {
      for (int jj = 0; jj < 32; ++jj) {
        const int64_t col = col0 + j0 + jj;
        if (col < p.n_inst) p.u[col * p.n + row] = V(V_UP, j0 + jj);
      }
    }
  }
  // wind down: every tensor-memory read has completed before the release
  tc::tc_fence_before();
  __syncthreads();
  __syncwarp();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------------
template <int METHOD>
int set_smem_attr() {
  static std::once_flag once;
  static cudaError_t e = cudaSuccess;
  std::call_once(once,
                 [] { e = cudaFuncSetAttribute(eig_kernel<METHOD>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM); });
  return cuda_check(e, "cudaFuncSetAttribute (dense eigenbasis kernel)");
}

template <int METHOD>
int launch(const CUtensorMap& tmA, const Params& p, unsigned grid, cudaStream_t s) {
  const int rc = set_smem_attr<METHOD>();
  if (rc) return rc;
  eig_kernel<METHOD><<<grid, THREADS, SMEM, s>>>(tmA, p);
  return cuda_check(cudaGetLastError(), "rk_dense_eig_evolve launch");
}

}  // namespace dense_eig
}  // namespace rk

using namespace rk;
using namespace rk::dense_eig;

extern "C" int64_t rk_dense_eig_work_bytes(int64_t n_inst) {
  if (n_inst < 1) return 0;
  return layout(n_inst).total;
}

extern "C" int rk_dense_eig_evolve(const rk_dense_eig_batch* b, void* stream) {
  if (!b || !b->state || !b->u || !b->work || !b->eig || !b->S || !b->Sinv || !b->shift || b->n_inst < 1) {
    set_error("rk_dense_eig_evolve: invalid batch");
    return RK_E_ARG;
  }
  if ((b->method != RK_ETD35 && b->method != RK_ETD34 && b->method != RK_IF34) || b->nl_kind != RK_NL_ALLEN_CAHN) {
    set_error("rk_dense_eig_evolve: the dense path implements ETD35, ETD34 and IF34 with the Allen-Cahn nonlinearity");
    return RK_E_UNSUPPORTED;
  }
  if (b->n < 1 || b->n > DM) {
    set_error("rk_dense_eig_evolve: n must be in 1..RK_DENSE_NMAX");
    return RK_E_ARG;
  }
  if ((reinterpret_cast<uintptr_t>(b->work) & 1023) != 0) {
    set_error("rk_dense_eig_evolve: work must be 1024-byte aligned");
    return RK_E_ARG;
  }
  if (b->max_attempts < 1) return RK_OK;
  const Layout L = layout(b->n_inst);
  unsigned char* w = static_cast<unsigned char*>(b->work);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = RK_OK;
  Params p{};
  p.st = b->state;
  p.A = reinterpret_cast<const float*>(w + L.a);
  p.V = reinterpret_cast<float*>(w + L.v);
  p.C = reinterpret_cast<float*>(w + L.c);
  p.eig = reinterpret_cast<const double*>(w + L.eig);
  p.shift = reinterpret_cast<const float*>(w + L.shift);
  p.u = b->u;
  p.n_inst = b->n_inst;
  p.bpad = L.bpad;
  p.n = b->n;
  p.err_eigen = b->err_eigen ? 1 : 0;
  p.first = b->first ? 1 : 0;
  p.max_attempts = b->max_attempts;
  p.ctl = b->ctl;
  p.ec = EtdCfg{b->etd.modecutoff, b->etd.contour_radius, b->etd.contour_points};
  if (p.first) {
    setup_kernel<<<(DM * DM + 255) / 256, 256, 0, s>>>(reinterpret_cast<float*>(w + L.a),
                                                       reinterpret_cast<double*>(w + L.eig),
                                                       reinterpret_cast<float*>(w + L.shift), b->n, b->eig, b->S,
                                                       b->Sinv, b->shift);
    rc = cuda_check(cudaGetLastError(), "rk_dense_eig_evolve set-up launch");
    if (rc) return rc;
  }
  CUtensorMap tmA;
  rc = make_tmap_f32_sw128(&tmA, p.A, DM, 2 * 2 * DM, DM);
  if (rc) return rc;
  const unsigned grid = (unsigned)(L.bpad / NT);
  rc = b->method == RK_ETD35   ? launch<RK_ETD35>(tmA, p, grid, s)
       : b->method == RK_ETD34 ? launch<RK_ETD34>(tmA, p, grid, s)
                               : launch<RK_IF34>(tmA, p, grid, s);
  if (rc) return rc;
  return cuda_check(cudaStreamSynchronize(s), "rk_dense_eig_evolve");
}
