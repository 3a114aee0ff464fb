// Dense (non-diagonal) operator path: ETD35 for a batch of instances that share one n x n
// lin_op (n <= 128), on the fifth-generation tensor cores.
//
// Replaces rkstiff/etd35.py:_Etd35NonDiagonal (etd35.py:498-720).  Per attempt, two
// kernels, each a no-op once the batch has left RK_ST_RUNNING (so a fixed launch sequence
// can run ahead of the host):
//   coef_kernel     when h changed: every block evaluates the 21 diagonal ETD35 coefficient
//                   functions of h * eig in FP64 (the reference's diagonalized arithmetic,
//                   etd35.py:348-495, with its contour mean for small |z|) and forms one tile
//                   of one matrix M_c = S diag(c) S^-1 in FP64 (the psi-matrices of
//                   etd35.py:602-658), stored as a TF32 hi/lo pair
//   attempt_kernel  one CTA per 64 instances: the ETD35 stages (etd35.py:690-720) as six
//                   K-concatenated GEMM chains, e.g. k3 = [E14 a31 a32] [u; N1; N2], run as
//                   3xTF32 tcgen05.mma (A_lo B_hi + A_hi B_lo + A_hi B_hi, FP32 accumulate in
//                   tensor memory) fed by TMA through a 4-slot mbarrier ring; the Allen-Cahn
//                   nonlinearity, the stage combinations, the new state and the per-instance
//                   error test (solveras.py:412-455) run in the epilogues; the last CTA to
//                   finish puts the batch's smallest s through the reference's accept/reject
//                   rule (solveras.py:457-554): the batch steps in lockstep
//
// Vectors live in global memory instance-major (each instance's 128 values contiguous, K
// innermost for the B operand) as FP32 hi/lo pairs; the working set (11 vectors x 8192
// instances x 1 KB) stays in L2.  Rows n..127 of every matrix and vector are zero.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cmath>
#include <mutex>
#include <string>

#include "rk_evolve.cuh"
#include "rk_launch.h"
#include "rk_tc.cuh"

namespace rk {
namespace dense {

constexpr int DM = RK_DENSE_NMAX;  // vector length (padded) = MMA M
constexpr int NT = RK_DENSE_TILE;  // instances per CTA = MMA N
constexpr int KC = 32;             // K elements per pipeline chunk (128 bytes of FP32)
constexpr int NS = 4;              // pipeline slots
constexpr int NCOEF = C35_N;       // 21 coefficient matrices
constexpr int C_ERR_EIG = NCOEF;   // diag(a75) S^-1: the error product in the eigenbasis
constexpr int NMAT = NCOEF + 1;
constexpr int A_TILE = DM * KC * 4;
constexpr int B_TILE = NT * KC * 4;
constexpr int SLOT_BYTES = 2 * A_TILE + 2 * B_TILE;
constexpr uint64_t WAIT_NS = 200000000ull;  // give up a wait after 200 ms
constexpr int GEMM_THREADS = 128;
// attempt kernel: warps 0-3 epilogues (one tensor-memory lane quarter each), warp 4 issues
// the MMAs, warp 5 the TMA loads
constexpr int ATTEMPT_THREADS = 192;
constexpr int MMA_TID = 128, PRODUCER_TID = 160;
constexpr int ATTEMPT_SMEM = 1024 + NS * SLOT_BYTES + 256;
constexpr int TMEM_COLS = 256;  // accumulator slots at columns 0 and NT, the error product at 2 NT

// N1 and N1B are N(u) of the state in U0 and U1: the last epilogue of an attempt writes
// N(unew) next to unew, so an attempt starts with N1 ready
enum { V_U0, V_U1, V_N1, V_N1B, V_N2, V_N3, V_N4, V_N5, V_N6, V_D23, V_D24, V_EV, NVEC };

struct Layout {  // byte offsets into the work buffer
  int64_t bpad, a, v, cd, eig, S, Si, shift, s, cmin, ctr, total;
};
RK_HD int64_t al1k(int64_t x) { return (x + 1023) & ~int64_t(1023); }
inline Layout layout(int64_t n_inst) {
  Layout L;
  L.bpad = (n_inst + NT - 1) / NT * NT;
  int64_t o = 0;
  L.a = o;
  o = al1k(o + (int64_t)NMAT * 2 * DM * DM * 4);
  L.v = o;
  o = al1k(o + (int64_t)NVEC * 2 * L.bpad * DM * 4);
  L.cd = o;
  o = al1k(o + (int64_t)NCOEF * DM * 8);
  L.eig = o;
  o = al1k(o + (int64_t)DM * 16);
  L.S = o;
  o = al1k(o + (int64_t)DM * DM * 8);
  L.Si = o;
  o = al1k(o + (int64_t)DM * DM * 8);
  L.shift = o;
  o = al1k(o + (int64_t)DM * 4);
  L.s = o;
  o = al1k(o + L.bpad * 8);
  L.cmin = o;
  o = al1k(o + (L.bpad / NT) * 8);
  L.ctr = o;
  o = al1k(o + 64);
  L.total = o;
  return L;
}

struct Params {
  rk_dense_state* st;
  float* A;              // [NMAT][2][DM][DM]
  float* V;              // [NVEC][2][bpad][DM]
  double* Cd;            // [NCOEF][DM]
  const cx<double>* eig; // [DM]
  const double* S;       // [DM][DM]
  const double* Si;      // [DM][DM]
  const float* shift;    // [DM]
  double* s;             // [bpad]
  double* cmin;          // [bpad / NT] smallest s of each CTA's instances (NaN: any NaN)
  unsigned int* ctr;     // CTAs of the current attempt that have finished
  int64_t n_inst, bpad;
  int n;
  int err_eigen;
  rk_controller ctl;
  EtdCfg ec;
};

RK_DEV float* vrow(const Params& p, int slot, int part, int64_t col) {
  return p.V + (((int64_t)slot * 2 + part) * p.bpad + col) * DM;
}
RK_DEV float vget(const Params& p, int slot, int64_t col, int row) {
  return vrow(p, slot, 0, col)[row] + vrow(p, slot, 1, col)[row];
}
RK_DEV void vput(const Params& p, int slot, int64_t col, int row, float v) {
  const float hi = tc::tf32_hi(v);
  vrow(p, slot, 0, col)[row] = hi;
  vrow(p, slot, 1, col)[row] = v - hi;
}
// Allen-Cahn nonlinearity in the lifted form (rkstiff/models.py:242-244)
RK_DEV float nl_ac(float w, float x) {
  const float v = w + x;
  return x - v * v * v;
}

// ---------------------------------------------------------------------------------
// set-up and state transfer
// ---------------------------------------------------------------------------------
__global__ void pad_kernel(Params p, const double* eig, const double* S, const double* Si, const double* shift) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < (int64_t)DM * DM) {
    const int r = (int)(i / DM), c = (int)(i % DM);
    const bool in = r < p.n && c < p.n;
    const_cast<double*>(p.S)[i] = in ? S[r * p.n + c] : 0.0;
    const_cast<double*>(p.Si)[i] = in ? Si[r * p.n + c] : 0.0;
  }
  if (i < DM) {
    const_cast<cx<double>*>(p.eig)[i] = cx<double>{i < p.n ? eig[i] : 0.0, 0.0};
    const_cast<float*>(p.shift)[i] = i < p.n ? (float)shift[i] : 0.f;
  }
  if (i < (int64_t)NCOEF * DM) p.Cd[i] = 0.0;
  if (i == 0) *p.ctr = 0u;
}

// caller's states (n_inst x n) into the current state vector, zero-padded
__global__ void load_u_kernel(Params p, const float* u) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.bpad * DM) return;
  const int64_t col = i / DM;
  const int row = (int)(i % DM);
  const float v = (col < p.n_inst && row < p.n) ? u[col * p.n + row] : 0.f;
  const int cur = p.st->cur;
  vput(p, cur ? V_U1 : V_U0, col, row, v);
  vput(p, cur ? V_N1B : V_N1, col, row, nl_ac(v, p.shift[row]));
}

__global__ void store_u_kernel(Params p, float* u) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n_inst * p.n) return;
  const int64_t col = i / p.n;
  const int row = (int)(i % p.n);
  u[i] = vget(p, p.st->cur ? V_U1 : V_U0, col, row);
}

// ---------------------------------------------------------------------------------
// coefficients (FP64)
// ---------------------------------------------------------------------------------
// When h differs from the h of the current matrices (exact compare, as etd35.py:851): every
// block evaluates the 21 diagonal coefficient functions of h * eig in FP64 into shared
// memory, then forms one 32 x 32 tile of one matrix M_c = S diag(c) S^-1.  h_coeff is
// advanced by the attempt that uses the matrices.
__global__ void __launch_bounds__(256) coef_kernel(Params p) {
  const rk_dense_state* st = p.st;
  if (st->status != RK_ST_RUNNING) return;
  const double h = st->h;
  if (h == st->h_coeff) return;
  __shared__ double Cd[NCOEF * DM];
  __shared__ double Ss[32][33];
  __shared__ double Sis[32][33];
  const int tid = threadIdx.x;
  for (int e = tid; e < NCOEF * DM; e += 256) Cd[e] = 0.0;
  __syncthreads();
  Group g{tid, 256, 0};
  compute_coeffs_impl<double, double, RK_ETD35, false>(g, p.n, DM, p.eig, Cd, h, p.ec);
  __syncthreads();
  const int c = blockIdx.y;
  const int i0 = (blockIdx.x >> 2) * 32, j0 = (blockIdx.x & 3) * 32;
  const int r = tid >> 3, q0 = (tid & 7) * 4;
  if (c == C_ERR_EIG) {
    // row i of S^-1 scaled by a75(h lambda_i)
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int i = i0 + r, j = j0 + q0 + t;
      const double v = Cd[C35_A75 * DM + i] * p.Si[i * DM + j];
      const float hi = tc::tf32_hi((float)v);
      p.A[(((int64_t)c * 2 + 0) * DM + i) * DM + j] = hi;
      p.A[(((int64_t)c * 2 + 1) * DM + i) * DM + j] = (float)(v - (double)hi);
    }
    return;
  }
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int k0 = 0; k0 < DM; k0 += 32) {
    for (int e = tid; e < 32 * 32; e += 256) {
      const int a = e >> 5, b = e & 31;
      Ss[a][b] = p.S[(i0 + a) * DM + k0 + b] * Cd[c * DM + k0 + b];
      Sis[a][b] = p.Si[(k0 + a) * DM + j0 + b];
    }
    __syncthreads();
#pragma unroll 8
    for (int k = 0; k < 32; ++k) {
      const double sv = Ss[r][k];
#pragma unroll
      for (int t = 0; t < 4; ++t) acc[t] += sv * Sis[k][q0 + t];
    }
    __syncthreads();
  }
#pragma unroll
  for (int t = 0; t < 4; ++t) {
    const int i = i0 + r, j = j0 + q0 + t;
    const float hi = tc::tf32_hi((float)acc[t]);
    p.A[(((int64_t)c * 2 + 0) * DM + i) * DM + j] = hi;
    p.A[(((int64_t)c * 2 + 1) * DM + i) * DM + j] = (float)(acc[t] - (double)hi);
  }
}

// ---------------------------------------------------------------------------------
// the tensor-core chain: D[acc] (+)= sum over chunks of A_chunk * B_chunk^T (3xTF32)
// ---------------------------------------------------------------------------------
struct ChunkCoord {
  int k0;              // K offset (elements) of the chunk
  int a_hi, a_lo;      // outer TMA coordinates of the A tiles (rows)
  int b_hi, b_lo;      // outer TMA coordinates of the B tiles (rows)
  int acc;             // accumulator (0: TMEM columns [0, NT), 1: [NT, 2 NT))
  int first;           // the chunk starts its accumulator's sum
};

struct Ring {
  unsigned char* sm;  // NS slots
  uint64_t* full;
  uint64_t* empty;
};

// The two roles of a chain, each run by one thread at the same time: the producer keeps the
// ring full (a slot is refilled once the MMAs that read it have completed), the MMA thread
// issues each chunk as soon as its tiles have landed.  `g` numbers chunks over the whole
// kernel (mbarrier parities); both roles advance it identically.  Return false when a wait
// timed out.
template <class ChunkFn>
RK_DEV bool chain_producer(int nch, ChunkFn chunk, int& g, const Ring& ring, const CUtensorMap* tmA,
                           const CUtensorMap* tmB) {
  for (int i = 0; i < nch; ++i) {
    const int gi = g + i, slot = gi % NS;
    if (gi >= NS && !tc::mbar_wait(&ring.empty[slot], (uint32_t)((gi / NS) - 1) & 1u, WAIT_NS)) return false;
    const ChunkCoord cc = chunk(i);
    unsigned char* base = ring.sm + slot * SLOT_BYTES;
    tc::mbar_arrive_expect_tx(&ring.full[slot], (uint32_t)SLOT_BYTES);
    tc::tma_load_2d(base, tmA, &ring.full[slot], cc.k0, cc.a_hi);
    tc::tma_load_2d(base + A_TILE, tmA, &ring.full[slot], cc.k0, cc.a_lo);
    tc::tma_load_2d(base + 2 * A_TILE, tmB, &ring.full[slot], cc.k0, cc.b_hi);
    tc::tma_load_2d(base + 2 * A_TILE + B_TILE, tmB, &ring.full[slot], cc.k0, cc.b_lo);
  }
  g += nch;
  return true;
}

template <class ChunkFn>
RK_DEV bool chain_mma(int nch, ChunkFn chunk, int& g, const Ring& ring, uint32_t tmem) {
  constexpr uint32_t idesc = tc::idesc_tf32(DM, NT);
  for (int i = 0; i < nch; ++i) {
    const int gi = g + i, slot = gi % NS;
    if (!tc::mbar_wait(&ring.full[slot], (uint32_t)(gi / NS) & 1u, WAIT_NS)) return false;
    tc::tc_fence_after();
    const ChunkCoord cc = chunk(i);
    const uint32_t sa = tc::smem_u32(ring.sm + slot * SLOT_BYTES);
    const uint64_t ahi = tc::sdesc_kmajor_sw128(sa), alo = tc::sdesc_kmajor_sw128(sa + A_TILE);
    const uint64_t bhi = tc::sdesc_kmajor_sw128(sa + 2 * A_TILE);
    const uint64_t blo = tc::sdesc_kmajor_sw128(sa + 2 * A_TILE + B_TILE);
    const uint32_t d = tmem + (uint32_t)(cc.acc * NT);
#pragma unroll
    for (int kk = 0; kk < KC / 8; ++kk) {
      const uint64_t o = (uint64_t)((kk * 32) >> 4);  // 8 TF32 = 32 bytes along K
      tc::mma_tf32(d, alo + o, bhi + o, idesc, (cc.first && kk == 0) ? 0u : 1u);
      tc::mma_tf32(d, ahi + o, blo + o, idesc, 1u);
      tc::mma_tf32(d, ahi + o, bhi + o, idesc, 1u);
    }
    tc::mma_commit(&ring.empty[slot]);
  }
  g += nch;
  return true;
}

// the accumulator rows of this thread's lane: NT FP32 values of columns [acc*NT, acc*NT+NT)
RK_DEV void load_acc(uint32_t tmem, int warp, int acc, float* v) {
  __syncwarp();  // tcgen05.ld is warp-collective
  const uint32_t base = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(acc * NT);
#pragma unroll
  for (int q = 0; q < NT / 16; ++q) tc::tmem_ld16(base + (uint32_t)(q * 16), v + q * 16);
  tc::tmem_ld_wait();
}

// 32 columns [half*32, half*32+32) of accumulator acc
RK_DEV void load_acc_half(uint32_t tmem, int warp, int acc, int half, float* v) {
  __syncwarp();
  const uint32_t base = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(acc * NT + half * 32);
  tc::tmem_ld16(base, v);
  tc::tmem_ld16(base + 16u, v + 16);
  tc::tmem_ld_wait();
}

struct Term {
  int coef, vec, acc;
};

// The reference's accept/reject rule (solveras.py:457-554) on the batch's smallest s; one
// thread, after every CTA of the attempt has written its instances' s.  h_coeff records
// the h the attempt's matrices were built for.
RK_DEV void apply_controller(const Params& p, double s) {
  rk_dense_state* st = p.st;
  const rk_controller& ctl = p.ctl;
  if (st->error) {
    st->status = RK_E_CUDA;  // a device wait timed out: stop (the host reports it)
    return;
  }
  const double h = st->h;
  if (h != st->h_coeff) {
    st->h_coeff = h;
    st->coeff_updates += 1;
  }
  st->attempts += 1;
  st->nl_evals += 5 + st->n1_fresh;
  st->s_last = s;
  if (isinf(s) || isnan(s) || s < 1.0) {
    st->accept = 0;
    st->n1_fresh = 0;
    st->rejects += 1;
    st->h = reject_h(s, h, ctl);
    st->numloops += 1;
    if (st->numloops > 50) st->status = RK_ST_MAX_LOOPS;
    else if (st->h < ctl.minh) st->status = RK_ST_MIN_STEP;
  } else {
    st->accept = 1;
    st->n1_fresh = 1;
    st->cur ^= 1;
    const double t = st->t + h;
    st->t = t;
    st->steps += 1;
    st->numloops = 0;
    const double hs = accept_h(s, h, ctl);
    st->h_suggest = hs;
    const double hn = (t + hs > st->tf) ? st->tf - t : hs;
    st->h = hn;
    if (!(t < st->tf)) st->status = RK_ST_DONE;
    else if (t + hn == t) st->status = RK_ST_MIN_STEP;
  }
}

// ---------------------------------------------------------------------------------
// one ETD35 attempt for NT instances
// ---------------------------------------------------------------------------------
// rkstiff/etd35.py:690-719 as GEMM chains (coefficient matrix, vector, accumulator), the
// terms that need the previous chain's epilogue last: while epilogue c runs on accumulator
// slot c % 2, chain c + 1 accumulates its other terms in the other slot.
struct ChainDef {
  Term t[7];
  int n;     // terms
  int ndep;  // trailing terms that read the previous epilogue's outputs
};

__global__ void __launch_bounds__(ATTEMPT_THREADS, 1)
    attempt_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmV, Params p) {
  rk_dense_state* st = p.st;
  if (st->status != RK_ST_RUNNING) return;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + NS * SLOT_BYTES);
  uint64_t* empty = full + NS;
  uint64_t* accb = empty + NS;  // chain c's accumulator complete (one phase per chain)
  uint64_t* epi = accb + 1;     // [2] epilogue c done (outputs written, slot c % 2 read): epi[c % 2]
  uint64_t* xb = epi + 2;       // exchanges among the epilogue threads (bounded, unlike bar.sync)
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(xb + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int tid = threadIdx.x, warp = tid >> 5, row = tid;
  const int64_t col0 = (int64_t)blockIdx.x * NT;
  const int cur = st->cur;
  const int vU = cur ? V_U1 : V_U0, vUN = cur ? V_U0 : V_U1;
  const int vN1 = cur ? V_N1B : V_N1, vN1N = cur ? V_N1 : V_N1B;

  if (tid == 0) {
    for (int i = 0; i < NS; ++i) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    tc::mbar_init(accb, 1);
    tc::mbar_init(&epi[0], 128);
    tc::mbar_init(&epi[1], 128);
    tc::mbar_init(xb, 128);
    *abort_flag = 0;
    tc::fence_mbar_init();
    tc::prefetch_tmap(&tmA);
    tc::prefetch_tmap(&tmV);
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
  const Ring ring{sm, full, empty};

  const ChainDef chains[6] = {
      {{{C35_E14, vU, 0}, {C35_A21, vN1, 0}}, 2, 0},
      {{{C35_E14, vU, 1}, {C35_A31, vN1, 1}, {C35_A32, V_N2, 1}}, 3, 1},
      {{{C35_E12, vU, 0}, {C35_A41, vN1, 0}, {C35_A43, V_N3, 0}}, 3, 1},
      {{{C35_E34, vU, 1}, {C35_A51, vN1, 1}, {C35_A52, V_D23, 1}, {C35_A54, V_N4, 1}}, 4, 1},
      {{{C35_E, vU, 0}, {C35_A61, vN1, 0}, {C35_A62, V_D24, 0}, {C35_A63, V_N3, 0}, {C35_A65, V_N5, 0}}, 5, 1},
      {{{C35_E, vU, 1}, {C35_A71, vN1, 1}, {C35_A73, V_N3, 1}, {C35_A74, V_N4, 1}, {C35_A75, V_N5, 1},
        {C35_A76, V_N6, 1}, {p.err_eigen ? C_ERR_EIG : C35_A75, V_EV, 2}},
       7,
       2}};

  auto chunk_of = [&](const ChainDef& cd, int i) {
    const Term& t = cd.t[i >> 2];
    ChunkCoord cc;
    cc.k0 = (i & 3) * KC;
    cc.a_hi = (t.coef * 2) * DM;
    cc.a_lo = (t.coef * 2 + 1) * DM;
    cc.b_hi = (int)((t.vec * 2) * p.bpad + col0);
    cc.b_lo = (int)((t.vec * 2 + 1) * p.bpad + col0);
    cc.acc = t.acc;
    cc.first = (i & 3) == 0 && ((i >> 2) == 0 || cd.t[(i >> 2) - 1].acc != t.acc);
    return cc;
  };

  if (tid == PRODUCER_TID) {
    // TMA loads of every chain, in order; a chain's trailing terms wait for the previous
    // epilogue (its outputs are in global memory, fenced for the async proxy)
    int g = 0;
    for (int c = 0; c < 6 && !*abort_flag; ++c) {
      const ChainDef& cd = chains[c];
      const int nind = (cd.n - cd.ndep) * (DM / KC), nch = cd.n * (DM / KC);
      auto ck = [&](int i) { return chunk_of(cd, i); };
      int gi = g;
      bool ok = chain_producer(nind, ck, gi, ring, &tmA, &tmV);
      if (ok && c > 0) ok = tc::mbar_wait(&epi[(c - 1) & 1], (uint32_t)(((c - 1) >> 1) & 1), WAIT_NS);
      if (ok) {
        auto ckd = [&](int i) { return chunk_of(cd, nind + i); };
        ok = chain_producer(nch - nind, ckd, gi, ring, &tmA, &tmV);
      }
      g = gi;
      if (!ok) {
        atomicOr(&st->error, 1);
        *abort_flag = 1;
      }
    }
  } else if (tid == MMA_TID) {
    int g = 0;
    for (int c = 0; c < 6; ++c) {
      const ChainDef& cd = chains[c];
      const int nch = cd.n * (DM / KC);
      bool ok = !*abort_flag;
      // the slot this chain accumulates in was read by epilogue c - 2
      if (ok && c >= 2) ok = tc::mbar_wait(&epi[c & 1], (uint32_t)(((c - 2) >> 1) & 1), WAIT_NS);
      if (ok) {
        tc::tc_fence_after();
        auto ck = [&](int i) {
          ChunkCoord cc = chunk_of(cd, i);
          cc.acc = cd.t[i >> 2].acc == 2 ? 2 : (c & 1);
          return cc;
        };
        ok = chain_mma(nch, ck, g, ring, tmem);
      }
      if (!ok) {
        atomicOr(&st->error, 1);
        *abort_flag = 1;
      }
      tc::mma_commit(accb);  // arrives once every MMA issued so far has completed
    }
  } else if (warp < 4) {
    // epilogues.  ev accumulates the error combination -N1 + 4 N3 - 6 N4 + 4 N5 - N6
    // (etd35.py:344) as the stages arrive and n2 keeps N2 for N2 - N3 and N2 - 3 N4 / 2,
    // so no epilogue reads a stage vector back.
    const float xr = p.shift[row];
    float ev[NT], n2[NT], acc[32];
    // all epilogue threads meet; a thread that gave up on an earlier wait never arrives, so
    // the others time out here instead of waiting forever
    int xphase = 0;
    auto sync_epi = [&]() -> bool {
      tc::mbar_arrive(xb);
      const bool w = tc::mbar_wait(xb, (uint32_t)xphase & 1u, WAIT_NS);
      ++xphase;
      if (!w) {
        atomicOr(&st->error, 2);
        *abort_flag = 1;
      }
      return w;
    };
#pragma unroll 16
    for (int j = 0; j < NT; ++j) ev[j] = -vget(p, vN1, col0 + j, row);
    for (int c = 0; c < 6; ++c) {
      if (!tc::mbar_wait(accb, (uint32_t)c & 1u, WAIT_NS)) {
        atomicOr(&st->error, 2);
        *abort_flag = 1;
      }
      if (*abort_flag) break;
      tc::tc_fence_after();
      const int slot = c & 1;
      if (c < 5) {
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          load_acc_half(tmem, warp, slot, half, acc);
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) {
            const int j = half * 32 + jj;
            const int64_t col = col0 + j;
            const float nk = nl_ac(acc[jj], xr);
            if (c == 0) {
              vput(p, V_N2, col, row, nk);
              n2[j] = nk;
            } else if (c == 1) {
              vput(p, V_N3, col, row, nk);
              vput(p, V_D23, col, row, n2[j] - nk);
              ev[j] = ev[j] + 4.f * nk;
            } else if (c == 2) {
              vput(p, V_N4, col, row, nk);
              vput(p, V_D24, col, row, n2[j] - (3.f * nk) * 0.5f);
              ev[j] = ev[j] - 6.f * nk;
            } else if (c == 3) {
              vput(p, V_N5, col, row, nk);
              ev[j] = ev[j] + 4.f * nk;
            } else {
              vput(p, V_N6, col, row, nk);
              vput(p, V_EV, col, row, ev[j] - nk);
            }
          }
        }
        tc::fence_proxy_async_global();
        tc::tc_fence_before();
        tc::mbar_arrive(&epi[slot]);
      } else {
        // new state, N(unew) for the next attempt, and the per-instance error test on the
        // new state (solveras.py:412-455).  The ring is idle: every chunk has been consumed.
        constexpr int LD = NT + 1;
        float* ru = reinterpret_cast<float*>(sm);
        float* re = ru + DM * LD;
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          float err[32];
          load_acc_half(tmem, warp, slot, half, acc);
          load_acc_half(tmem, warp, 2, half, err);
#pragma unroll
          for (int jj = 0; jj < 32; ++jj) {
            const int j = half * 32 + jj;
            vput(p, vUN, col0 + j, row, acc[jj]);
            vput(p, vN1N, col0 + j, row, nl_ac(acc[jj], xr));
            ru[row * LD + j] = acc[jj] * acc[jj];
            re[row * LD + j] = err[jj] * err[jj];
          }
        }
        tc::tc_fence_before();
        if (!sync_epi()) break;
        const int j = tid >> 1, half = tid & 1;
        float mx = 0.f;
        int nan = 0;
        for (int r = 64 * half; r < 64 * half + 64; ++r) {
          const float a2 = ru[r * LD + j];
          if (a2 != a2) nan = 1;
          else mx = fmaxf(mx, a2);
        }
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
        nan |= __shfl_xor_sync(0xffffffffu, nan, 1);
        const double maxu = nan ? nan_d() : (double)mx;
        // NaN keeps every comparison false, as in the reference
        const float thr = (float)(p.ctl.adapt_cutoff * p.ctl.adapt_cutoff * maxu);
        df au{0.f, 0.f}, ae{0.f, 0.f};
        for (int r = 64 * half; r < 64 * half + 64; ++r) {
          const float a2 = ru[r * LD + j];
          if (a2 > thr) {
            au = df_add(au, a2);
            ae = df_add(ae, re[r * LD + j]);
          }
        }
        au = df_add(au, df{__shfl_xor_sync(0xffffffffu, au.hi, 1), __shfl_xor_sync(0xffffffffu, au.lo, 1)});
        ae = df_add(ae, df{__shfl_xor_sync(0xffffffffu, ae.hi, 1), __shfl_xor_sync(0xffffffffu, ae.lo, 1)});
        double sv = INFINITY;  // padding columns do not take part
        if (col0 + j < p.n_inst) {
          const double su = (double)au.hi + (double)au.lo, se = (double)ae.hi + (double)ae.lo;
          const double ratio = (p.ctl.epsilon * p.ctl.epsilon * su) / se;
          if (ratio != ratio || isinf(ratio)) {
            sv = p.ctl.safety_f * ratio;
          } else {
            const float rf = (float)fmin(ratio, 1e30);
            sv = p.ctl.safety_f * (double)exp2f(log2f(rf) * (0.5f / 4.f));  // q = 4
          }
          if (half == 0) p.s[col0 + j] = sv;
        }
        // the CTA's smallest s (NaN if any is NaN) for the batch controller
        int snan = sv != sv;
        double smin = snan ? INFINITY : sv;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) smin = fmin(smin, __shfl_xor_sync(0xffffffffu, smin, o));
        snan = __any_sync(0xffffffffu, snan);
        __shared__ double cm[4];
        __shared__ int cn[4];
        if ((tid & 31) == 0) {
          cm[warp] = smin;
          cn[warp] = snan;
        }
        if (!sync_epi()) break;
        if (tid == 0) {
          for (int i = 1; i < 4; ++i) {
            smin = fmin(smin, cm[i]);
            snan |= cn[i];
          }
          p.cmin[blockIdx.x] = snan ? nan_d() : smin;
        }
      }
    }
  }
  // wind down: every TMEM read has completed (tcgen05.wait::ld) before the release
  tc::tc_fence_before();
  __syncthreads();
  __syncwarp();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, TMEM_COLS);
  }
  // The last CTA to finish applies the lockstep controller to the batch's smallest s.
  // Every CTA read the state before incrementing the counter, so the update cannot race
  // with a reader of this attempt.
  __shared__ int last;
  if (tid == 0) {
    __threadfence();
    last = atomicAdd(p.ctr, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  __shared__ double wmin[ATTEMPT_THREADS / 32];
  __shared__ int wnan[ATTEMPT_THREADS / 32];
  double m = INFINITY;
  int nan = 0;
  for (int i = tid; i < (int)gridDim.x; i += ATTEMPT_THREADS) {
    const double sv = __ldcg(p.cmin + i);
    if (sv != sv) nan = 1;
    else m = fmin(m, sv);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
  nan = __any_sync(0xffffffffu, nan);
  if ((tid & 31) == 0) {
    wmin[warp] = m;
    wnan[warp] = nan;
  }
  __syncthreads();
  if (tid == 0) {
    for (int i = 0; i < ATTEMPT_THREADS / 32; ++i) {
      m = fmin(m, wmin[i]);
      nan |= wnan[i];
    }
    apply_controller(p, nan ? nan_d() : m);
    *p.ctr = 0u;
    __threadfence();
  }
}

// ---------------------------------------------------------------------------------
// the standalone 3xTF32 product (check of the chain): D[N][DM] = B[N][K] A[DM][K]^T
// ---------------------------------------------------------------------------------
__global__ void split_kernel(const float* x, float* hi, float* lo, int64_t count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const float v = x[i];
  const float h = tc::tf32_hi(v);
  hi[i] = h;
  lo[i] = v - h;
}

__global__ void __launch_bounds__(GEMM_THREADS, 1)
    gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, float* D, int K,
                int N, int* error) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + NS * SLOT_BYTES);
  uint64_t* empty = full + NS;
  uint64_t* accb = empty + NS;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accb + 1);
  const int tid = threadIdx.x, warp = tid >> 5;
  const int col0 = blockIdx.x * NT;
  if (tid == 0) {
    for (int i = 0; i < NS; ++i) {
      tc::mbar_init(&full[i], 1);
      tc::mbar_init(&empty[i], 1);
    }
    tc::mbar_init(accb, 1);
    tc::fence_mbar_init();
  }
  __syncwarp();
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, 2 * NT);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  if (tid == 0 || tid == 32) {
    int g = 0;
    const Ring ring{sm, full, empty};
    auto chunk = [&](int i) {
      ChunkCoord cc;
      cc.k0 = i * KC;
      cc.a_hi = 0;
      cc.a_lo = DM;
      cc.b_hi = col0;
      cc.b_lo = N + col0;
      cc.acc = 0;
      cc.first = i == 0;
      return cc;
    };
    if (tid == 32) {
      if (!chain_producer(K / KC, chunk, g, ring, &tmA, &tmB)) atomicOr(error, 1);
    } else {
      if (!chain_mma(K / KC, chunk, g, ring, tmem)) atomicOr(error, 1);
      tc::mma_commit(accb);
    }
  }
  const bool ok = tc::mbar_wait(accb, 0u, WAIT_NS);
  if (!ok) atomicOr(error, 2);
  tc::tc_fence_after();
  __syncthreads();
  if (ok) {
    float acc[NT];
    load_acc(tmem, warp, 0, acc);
    for (int j = 0; j < NT; ++j) D[(int64_t)(col0 + j) * DM + tid] = acc[j];
  }
  tc::tc_fence_before();
  __syncthreads();
  __syncwarp();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 2 * NT);
  }
}

// ---------------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static std::once_flag once;
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// rows x inner FP32 matrix (row-major), box of 32 x box_rows, 128-byte swizzle
int make_map(CUtensorMap* m, const void* base, int64_t inner, int64_t rows, int box_rows) {
  auto fn = encode_fn();
  if (!fn) {
    set_error("cuTensorMapEncodeTiled is not available from the driver");
    return RK_E_CUDA;
  }
  const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)inner * 4};
  const cuuint32_t box[2] = {(cuuint32_t)KC, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
    return RK_E_CUDA;
  }
  return RK_OK;
}

int set_smem_attr() {
  static std::once_flag once;
  static cudaError_t e = cudaSuccess;
  std::call_once(once, [] {
    e = cudaFuncSetAttribute(attempt_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ATTEMPT_SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ATTEMPT_SMEM);
  });
  return cuda_check(e, "cudaFuncSetAttribute (dense kernels)");
}

}  // namespace dense

int make_tmap_f32_sw128(void* map, const void* base, int64_t inner, int64_t rows, int box_rows) {
  return dense::make_map(static_cast<CUtensorMap*>(map), base, inner, rows, box_rows);
}

}  // namespace rk

using namespace rk;
using namespace rk::dense;

extern "C" int64_t rk_dense_work_bytes(int64_t n_inst) {
  if (n_inst < 1) return 0;
  return layout(n_inst).total;
}

extern "C" int rk_dense_evolve(const rk_dense_batch* b, void* stream) {
  if (!b || !b->state || !b->u || !b->work || !b->eig || !b->S || !b->Sinv || !b->shift || b->n_inst < 1) {
    set_error("rk_dense_evolve: invalid batch");
    return RK_E_ARG;
  }
  if (b->method != RK_ETD35 || b->nl_kind != RK_NL_ALLEN_CAHN) {
    set_error("rk_dense_evolve: only ETD35 with the Allen-Cahn nonlinearity is built");
    return RK_E_UNSUPPORTED;
  }
  if (b->n < 1 || b->n > DM) {
    set_error("rk_dense_evolve: n must be in 1..128");
    return RK_E_SIZE;
  }
  if ((reinterpret_cast<uintptr_t>(b->work) & 1023) != 0) {
    set_error("rk_dense_evolve: work must be 1024-byte aligned");
    return RK_E_ARG;
  }
  const Layout L = layout(b->n_inst);
  if ((int64_t)NVEC * 2 * L.bpad > INT32_MAX / 2) {
    set_error("rk_dense_evolve: too many instances");
    return RK_E_SIZE;
  }
  if (int e = set_smem_attr()) return e;
  unsigned char* w = static_cast<unsigned char*>(b->work);
  Params p;
  p.st = b->state;
  p.A = reinterpret_cast<float*>(w + L.a);
  p.V = reinterpret_cast<float*>(w + L.v);
  p.Cd = reinterpret_cast<double*>(w + L.cd);
  p.eig = reinterpret_cast<const cx<double>*>(w + L.eig);
  p.S = reinterpret_cast<const double*>(w + L.S);
  p.Si = reinterpret_cast<const double*>(w + L.Si);
  p.shift = reinterpret_cast<const float*>(w + L.shift);
  p.s = reinterpret_cast<double*>(w + L.s);
  p.cmin = reinterpret_cast<double*>(w + L.cmin);
  p.ctr = reinterpret_cast<unsigned int*>(w + L.ctr);
  p.n_inst = b->n_inst;
  p.bpad = L.bpad;
  p.n = b->n;
  p.err_eigen = b->err_eigen ? 1 : 0;
  p.ctl = b->ctl;
  p.ec = EtdCfg{b->etd.modecutoff, b->etd.contour_radius, b->etd.contour_points};
  CUtensorMap tmA, tmV;
  if (int e = make_map(&tmA, p.A, DM, (int64_t)NMAT * 2 * DM, DM)) return e;
  if (int e = make_map(&tmV, p.V, DM, (int64_t)NVEC * 2 * L.bpad, NT)) return e;
  cudaStream_t s = (cudaStream_t)stream;
  pad_kernel<<<(DM * DM + 255) / 256, 256, 0, s>>>(p, b->eig, b->S, b->Sinv, b->shift);
  load_u_kernel<<<(unsigned)((L.bpad * DM + 255) / 256), 256, 0, s>>>(p, b->u);
  if (int e = cuda_check(cudaGetLastError(), "dense set-up launch")) return e;
  rk_dense_state hs;
  const int64_t per_check = 32;  // attempts between host reads of the state (no-op launches past the end are cheap)
  for (int64_t a = 0; a < b->max_attempts; a += per_check) {
    const int64_t r_end = a + per_check < b->max_attempts ? per_check : b->max_attempts - a;
    for (int64_t r = 0; r < r_end; ++r) {
      coef_kernel<<<dim3(16, NMAT), 256, 0, s>>>(p);
      attempt_kernel<<<(unsigned)(L.bpad / NT), ATTEMPT_THREADS, ATTEMPT_SMEM, s>>>(tmA, tmV, p);
    }
    if (int e = cuda_check(cudaGetLastError(), "dense attempt launch")) return e;
    if (int e = cuda_check(cudaMemcpyAsync(&hs, b->state, sizeof(hs), cudaMemcpyDeviceToHost, s), "state read")) return e;
    if (int e = cuda_check(cudaStreamSynchronize(s), "dense attempts")) return e;
    if (hs.status != RK_ST_RUNNING) break;
  }
  store_u_kernel<<<(unsigned)((b->n_inst * b->n + 255) / 256), 256, 0, s>>>(p, b->u);
  if (int e = cuda_check(cudaGetLastError(), "dense store launch")) return e;
  if (int e = cuda_check(cudaStreamSynchronize(s), "dense store")) return e;
  if (hs.error) {
    set_error("rk_dense_evolve: a device wait timed out (error bits " + std::to_string(hs.error) + ")");
    return RK_E_CUDA;
  }
  return RK_OK;
}

extern "C" int64_t rk_tf32x3_work_bytes(int64_t K, int64_t N) { return 2 * (DM * K + N * K) * 4 + 256; }

extern "C" int rk_tf32x3_gemm(const float* A, const float* B, float* D, int64_t K, int64_t N, void* work,
                              void* stream) {
  if (!A || !B || !D || !work || K < KC || K % KC || N < NT || N % NT || K > 4096 || N > (1 << 20)) {
    set_error("rk_tf32x3_gemm: K must be a positive multiple of 32 (<= 4096), N of 64");
    return RK_E_ARG;
  }
  if ((reinterpret_cast<uintptr_t>(work) & 255) != 0) {
    set_error("rk_tf32x3_gemm: work must be 256-byte aligned");
    return RK_E_ARG;
  }
  if (int e = set_smem_attr()) return e;
  float* Ahl = static_cast<float*>(work);
  float* Bhl = Ahl + 2 * DM * K;
  int* err = reinterpret_cast<int*>(Bhl + 2 * N * K);
  cudaStream_t s = (cudaStream_t)stream;
  split_kernel<<<(unsigned)((DM * K + 255) / 256), 256, 0, s>>>(A, Ahl, Ahl + DM * K, DM * K);
  split_kernel<<<(unsigned)((N * K + 255) / 256), 256, 0, s>>>(B, Bhl, Bhl + N * K, N * K);
  if (int e = cuda_check(cudaMemsetAsync(err, 0, sizeof(int), s), "memset")) return e;
  CUtensorMap tmA, tmB;
  if (int e = make_map(&tmA, Ahl, K, 2 * DM, DM)) return e;
  if (int e = make_map(&tmB, Bhl, K, 2 * N, NT)) return e;
  gemm_kernel<<<(unsigned)(N / NT), GEMM_THREADS, ATTEMPT_SMEM, s>>>(tmA, tmB, D, (int)K, (int)N, err);
  if (int e = cuda_check(cudaGetLastError(), "gemm launch")) return e;
  int herr = 0;
  if (int e = cuda_check(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, s), "error read")) return e;
  if (int e = cuda_check(cudaStreamSynchronize(s), "gemm")) return e;
  if (herr) {
    set_error("rk_tf32x3_gemm: a device wait timed out (error bits " + std::to_string(herr) + ")");
    return RK_E_CUDA;
  }
  return RK_OK;
}
