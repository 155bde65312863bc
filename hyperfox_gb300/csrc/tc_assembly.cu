// Element operator contractions on the tensor cores (tcgen05, sm_103a).
//
// Every block HyperFox's operators integrate over an element is a contraction
// over integration points of a per-element coefficient row with a reference
// table that is the same for all elements:
//
//   volume  X[r][j] = sum_q a_r(q) phi_j(q)       r over
//     C_d (Squ, HDGBase.cpp:67-158):    a = dV (J^{-1} grad phi_i)_d
//     K_d (Suq volume, HDGDiffusion.cpp:74-145): a = dV (kappa J^{-1} grad phi_i)_d
//     M   (Sqq, Mass.cpp:5-38):          a = dV phi_i
//   face    Y[r][b] = sum_k c_r(k) fphi_b(k)      r over
//     T   (tau face mass, HDGBase.cpp:95-120): c = dS tau fphi_a
//     E_d (n phi phi, HDGBase.cpp:121-140):    c = dS n_d fphi_a
//     H_d (kappa n phi phi, HDGDiffusion.cpp:110-145): c = dS (kappa n)_d fphi_a
//
// i.e. B^T diag(w J) B with B the reference basis. One CTA of 128 threads takes
// one element at a time: its threads compute the coefficient rows (geometry in
// FP32 from the FP64 mesh) into shared memory as 128-row MMA tiles, one thread
// issues tcgen05.mma (kind::tf32, M = 128, FP32 accumulation in TMEM), and the
// four warps drain the accumulator rows with tcgen05.ld and write them to HBM
// with coalesced stores. The reference tables (the B operands and the FP32 basis
// tables for the geometry) are staged once per CTA by one cp.async.bulk copy.
//
// Precision: both operands are split into TF32 high and low parts (x = hi + lo,
// each a TF32 value) and every product is accumulated as hi*hi + hi*lo + lo*hi,
// which keeps about 21 significant bits per product (the lo*lo term, 2^-22
// relative, is dropped); the FP32 accumulation adds 2^-24 per term. The blocks
// agree with the FP64 quadrature to about 1e-6 of their largest entry; the
// stated bound (tested against the FP64 oracle) is 2e-5.
//
// Output per element (FP32, contiguous): the volume rows [C_0..C_{D-1} | K_0..
// K_{D-1} | M] of N values each, the face rows [T | E | H] of NF values each, and
// the source load f_u (N values, Source.cpp:24-48). Index conventions are those
// of the FP32 element kernel that consumes them (hdg_local.cu).
//
// Every wait on an mbarrier is bounded: a wait that runs out sets status 2 and
// the CTA stops, frees its TMEM and returns.
#include <cstdint>
#include <cstring>
#include <vector>

#include "cg_operators.h"
#include "hfx_device.h"
#include "tc_assembly.h"

namespace hfx {
namespace {

constexpr int kThreads = 128;
constexpr uint32_t kWaitLimit = 1u << 26;  // mbarrier polls before a wait is abandoned

template <int D, int P>
struct TcDims {
  using K = Dims<D, P>;
  static constexpr int N = K::N, NF = K::NF, F = K::F, NI = K::NI, NIF = K::NIF, DM = D - 1;
  static constexpr int NIP = (NI + 7) / 8 * 8;    // K of the volume MMAs (tf32: 8 per instruction)
  static constexpr int NIFP = (NIF + 7) / 8 * 8;  // K of the face MMAs
  static constexpr int NVB = 32;                  // N of the volume MMAs (N <= 32 nodes)
  static constexpr int NFB = 16;                  // N of the face MMAs (NF <= 16)
  static constexpr int RV = 2 * D * N + N;        // volume rows: C_d, K_d, M
  static constexpr int RF = F * NF * (1 + 2 * D); // face rows: T, E_d, H_d
  static constexpr int TV = (RV + 127) / 128;     // 128-row tiles
  static constexpr int TF = (RF + 127) / 128;
  static constexpr int A_FLOATS = (TV * 128 * NIP > TF * 128 * NIFP) ? TV * 128 * NIP : TF * 128 * NIFP;
  static constexpr int TMEM_COLS_USED = TV * NVB + TF * NFB;
  static constexpr int TMEM_COLS = TMEM_COLS_USED <= 32 ? 32 : TMEM_COLS_USED <= 64 ? 64 : TMEM_COLS_USED <= 128 ? 128 : 256;
  // packed FP32 table (host image, copied as one block): B images then the basis tables
  static constexpr int TB_VHI = 0;
  static constexpr int TB_VLO = TB_VHI + NVB * NIP;
  static constexpr int TB_FHI = TB_VLO + NVB * NIP;
  static constexpr int TB_FLO = TB_FHI + NFB * NIFP;
  static constexpr int TB_PHI = TB_FLO + NFB * NIFP;
  static constexpr int TB_DPHI = TB_PHI + NI * N;
  static constexpr int TB_W = TB_DPHI + NI * N * D;
  static constexpr int TB_FPHI = TB_W + NI;
  static constexpr int TB_FDPHI = TB_FPHI + NIF * NF;
  static constexpr int TB_FW = TB_FDPHI + NIF * NF * DM;
  static constexpr int TB_END = TB_FW + NIF;
  static constexpr int TB_FLOATS = (TB_END + 3) / 4 * 4;  // bulk copies move multiples of 16 bytes
  // per-element scratch (floats)
  static constexpr int S_X = 0;
  static constexpr int S_KAP = S_X + N * D;
  static constexpr int S_TAU = S_KAP + N * D * D;
  static constexpr int S_DV = S_TAU + F * NF;
  static constexpr int S_IJ = S_DV + NI;           // dV J^{-1}, [NI][D][D]
  static constexpr int S_KIJ = S_IJ + NI * D * D;  // dV kappa J^{-1}, [NI][D][D]
  static constexpr int S_FQ = S_KIJ + NI * D * D;
  static constexpr int S_DST = S_FQ + NI;
  static constexpr int S_DSN = S_DST + F * NIF;
  static constexpr int S_DSKN = S_DSN + F * NIF * D;
  static constexpr int S_END = S_DSKN + F * NIF * D;
  static constexpr int S_FLOATS = (S_END + 3) / 4 * 4;
  // dynamic shared memory: A hi, A lo (1024-aligned), tables, scratch
  static constexpr size_t OFF_AHI = 0;
  static constexpr size_t OFF_ALO = OFF_AHI + (size_t)A_FLOATS * 4;
  static constexpr size_t OFF_TAB = OFF_ALO + (size_t)A_FLOATS * 4;
  static constexpr size_t OFF_SCR = OFF_TAB + (size_t)TB_FLOATS * 4;
  static constexpr size_t SMEM = OFF_SCR + (size_t)S_FLOATS * 4 + 1024;  // + base alignment slack
  static constexpr int OUT_STRIDE = RV * N + RF * NF + N;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared memory matrix descriptor: K-major, no swizzle; core matrices of 8 rows x 16 bytes
// stored contiguously, lbo = bytes between core matrices adjacent in K, sbo = bytes between
// core matrices adjacent in M/N (the next 8 rows)
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of sm_100-class tensor cores
  return d;
}

// instruction descriptor: D FP32, A and B TF32, both K-major, N >> 3, M >> 4
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// element (r, k) of a K-major operand with kc = K/4 chunks of 16 bytes per row: core matrix
// (r/8, k/4) at ((r/8) kc + k/4) * 32 floats, row r%8 at +4 (r%8), element k%4
__host__ __device__ __forceinline__ int cm_index(int r, int k, int kc) {
  return ((r >> 3) * kc + (k >> 2)) * 32 + (r & 7) * 4 + (k & 3);
}

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t u;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(u) : "f"(x));
  return __uint_as_float(u);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p; }" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// bounded wait on an mbarrier phase; false if it ran out
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) {
  uint32_t done = 0;
  for (uint32_t it = 0; it < kWaitLimit && !done; ++it)
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
  return done != 0;
}

template <int NCOL>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, float* v);

template <>
__device__ __forceinline__ void tmem_ld<32>(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int c = 0; c < 32; ++c) v[c] = __uint_as_float(r[c]);
}

template <>
__device__ __forceinline__ void tmem_ld<16>(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int c = 0; c < 16; ++c) v[c] = __uint_as_float(r[c]);
}

// Issue the hi/lo-split MMAs of `tiles` 128-row tiles with K = kp (tf32: 8 per
// instruction) against one B image of nb rows; accumulators at tmem + t * nb.
__device__ __forceinline__ void issue_tiles(uint32_t tmem, int tiles, int kp, int nb, uint32_t aHi, uint32_t aLo,
                                            uint32_t bHi, uint32_t bLo) {
  const uint32_t kc = (uint32_t)kp / 4;
  const uint32_t sbo = kc * 128u, lbo = 128u;
  const uint32_t idesc = idesc_tf32(128, nb);
  for (int t = 0; t < tiles; ++t) {
    const uint32_t aoff = (uint32_t)t * 128u * (uint32_t)kp * 4u;
    const uint32_t td = tmem + (uint32_t)(t * nb);
    for (int s = 0; s < kp / 8; ++s) {
      const uint32_t ks = (uint32_t)s * 256u;  // two 16-byte chunks per K step
      const uint64_t ah = smem_desc(aHi + aoff + ks, lbo, sbo), al = smem_desc(aLo + aoff + ks, lbo, sbo);
      const uint64_t bh = smem_desc(bHi + ks, lbo, sbo), bl = smem_desc(bLo + ks, lbo, sbo);
      mma_tf32(td, ah, bh, idesc, s > 0 ? 1u : 0u);
      mma_tf32(td, ah, bl, idesc, 1u);
      mma_tf32(td, al, bh, idesc, 1u);
    }
  }
}

template <int D, int P>
__global__ void __launch_bounds__(kThreads) tc_element_blocks(TcBlockParams p) {
  using T = TcDims<D, P>;
  constexpr int N = T::N, NF = T::NF, F = T::F, NI = T::NI, NIF = T::NIF, DM = T::DM;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  float* aHi = (float*)(smem + T::OFF_AHI);
  float* aLo = (float*)(smem + T::OFF_ALO);
  float* tab = (float*)(smem + T::OFF_TAB);
  float* scr = (float*)(smem + T::OFF_SCR);
  __shared__ __align__(8) uint64_t bars[2];  // 0: table copy, 1: MMA completion
  __shared__ uint32_t tmemBase;
  __shared__ int sFaceNodes[F * NF];
  __shared__ int sOpp[F];
  __shared__ int sAbort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[1])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    sAbort = 0;
  }
  for (int i = tid; i < F * NF; i += kThreads) sFaceNodes[i] = p.itab[i];
  for (int i = tid; i < F; i += kThreads) sOpp[i] = p.itab[F * NF + i];
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmemBase)),
                 "r"((uint32_t)T::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmemBase;
  // stage the packed table once per CTA (one bulk copy, completion counted in bytes)
  if (tid == 0) {
    const uint32_t bytes = (uint32_t)T::TB_FLOATS * 4u;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&bars[0])), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(tab)),
                 "l"(p.tctab), "r"(bytes), "r"(smem_u32(&bars[0]))
                 : "memory");
  }
  if (!mbar_wait(&bars[0], 0)) {
    atomicCAS(p.status, 0, 2);
    sAbort = 1;
  }
  __syncthreads();
  const float* phi = tab + T::TB_PHI;
  const float* dphi = tab + T::TB_DPHI;
  const float* w = tab + T::TB_W;
  const float* fphi = tab + T::TB_FPHI;
  const float* fdphi = tab + T::TB_FDPHI;
  const float* fw = tab + T::TB_FW;
  float* X = scr + T::S_X;
  float* kapN = scr + T::S_KAP;
  float* tauL = scr + T::S_TAU;
  float* dV = scr + T::S_DV;
  float* IJ = scr + T::S_IJ;
  float* KIJ = scr + T::S_KIJ;
  float* fq = scr + T::S_FQ;
  float* dSt = scr + T::S_DST;
  float* dSn = scr + T::S_DSN;
  float* dSkn = scr + T::S_DSKN;
  const uint32_t aHiS = smem_u32(aHi), aLoS = smem_u32(aLo);
  const uint32_t tabS = smem_u32(tab);
  uint32_t phase = 0;

  for (int64_t e = blockIdx.x; e < p.nCells && !sAbort; e += gridDim.x) {
    float* out = p.out + e * (int64_t)T::OUT_STRIDE;
    // ---------------------------------------------------------------- gather
    const int* cell = p.cells + e * N;
    for (int i = tid; i < N * D; i += kThreads) X[i] = (float)p.coords[(int64_t)cell[i / D] * D + (i % D)];
    for (int i = tid; i < N * D * D; i += kThreads) {
      const int n = i / (D * D), a = i % (D * D);
      float v;
      if (p.kc == 0) v = (a % (D + 1) == 0) ? 1.f : 0.f;
      else {
        const int64_t bk = p.kappaLayout == 0 ? (int64_t)cell[n] * p.kc : (e * N + n) * p.kc;
        v = p.kc == 1 ? ((a % (D + 1) == 0) ? (float)p.kappa[bk] : 0.f) : (float)p.kappa[bk + a];
      }
      kapN[i] = v;
    }
    for (int i = tid; i < F * NF; i += kThreads) {
      const int f = p.cell2face[e * F + i / NF];
      const int side = (p.face2cell[2 * (int64_t)f] == (int)e) ? 0 : 1;
      const int q = p.perm[e * F * NF + i];
      tauL[i] = (float)p.tau[((int64_t)f * NF + q) * p.tauVals + (p.tauVals == 2 ? side : 0)];
    }
    __syncthreads();
    // ------------------------------------------------ volume and face geometry
    for (int q = tid; q < NI; q += kThreads) {
      float J[D][D];
      for (int r = 0; r < D; ++r)
        for (int s = 0; s < D; ++s) {
          float acc = 0.f;
          for (int i = 0; i < N; ++i) acc += dphi[(q * N + i) * D + r] * X[i * D + s];
          J[r][s] = acc;
        }
      float det, iv[D][D];
      if (D == 2) {
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const float id = 1.f / det;
        iv[0][0] = J[1][1] * id;
        iv[0][1] = -J[0][1] * id;
        iv[1][0] = -J[1][0] * id;
        iv[1][1] = J[0][0] * id;
      } else {
        const float c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const float c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const float c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        const float id = 1.f / det;
        iv[0][0] = c00 * id;
        iv[1][0] = c01 * id;
        iv[2][0] = c02 * id;
        iv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
        iv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
        iv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
        iv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
        iv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
        iv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
      }
      const float dv = w[q] * det;
      dV[q] = dv;
      float kq[D][D];  // kappa at the IP, column-major nodal storage: (a, b) at a + b D
      for (int a = 0; a < D; ++a)
        for (int b = 0; b < D; ++b) {
          float acc = 0.f;
          for (int i = 0; i < N; ++i) acc += phi[q * N + i] * kapN[i * D * D + a + b * D];
          kq[a][b] = acc;
        }
      for (int a = 0; a < D; ++a)
        for (int c = 0; c < D; ++c) {
          IJ[(q * D + a) * D + c] = dv * iv[a][c];
          float acc = 0.f;
          for (int b = 0; b < D; ++b) acc += kq[a][b] * iv[b][c];
          KIJ[(q * D + a) * D + c] = dv * acc;
        }
      float fval = 0.f;
      if (p.srcMode == 1) fval = (float)p.src[e * NI + q];
      else if (p.srcMode == 2) {
        fval = (float)p.srcParam;
        for (int k = 0; k < D; ++k) {
          float xk = 0.f;
          for (int i = 0; i < N; ++i) xk += phi[q * N + i] * X[i * D + k];
          fval *= sinpif(xk);
        }
      }
      fq[q] = fval * dv;
    }
    for (int fk = tid; fk < F * NIF; fk += kThreads) {
      const int f = fk / NIF, k = fk % NIF;
      float Jf[D - 1][D];
      for (int r = 0; r < DM; ++r)
        for (int s = 0; s < D; ++s) {
          float acc = 0.f;
          for (int i = 0; i < NF; ++i) acc += fdphi[(k * NF + i) * DM + r] * X[sFaceNodes[f * NF + i] * D + s];
          Jf[r][s] = acc;
        }
      float nv[D], ds;
      if (D == 2) {
        ds = sqrtf(Jf[0][0] * Jf[0][0] + Jf[0][1] * Jf[0][1]);
        nv[0] = -Jf[0][1];
        nv[1] = Jf[0][0];
      } else {
        const float g00 = Jf[0][0] * Jf[0][0] + Jf[0][1] * Jf[0][1] + Jf[0][2] * Jf[0][2];
        const float g11 = Jf[1][0] * Jf[1][0] + Jf[1][1] * Jf[1][1] + Jf[1][2] * Jf[1][2];
        const float g01 = Jf[0][0] * Jf[1][0] + Jf[0][1] * Jf[1][1] + Jf[0][2] * Jf[1][2];
        ds = sqrtf(g00 * g11 - g01 * g01);
        nv[0] = Jf[0][1] * Jf[1][2] - Jf[0][2] * Jf[1][1];
        nv[1] = Jf[0][2] * Jf[1][0] - Jf[0][0] * Jf[1][2];
        nv[2] = Jf[0][0] * Jf[1][1] - Jf[0][1] * Jf[1][0];
      }
      float nn = 0.f;
      for (int a = 0; a < D; ++a) nn += nv[a] * nv[a];
      nn = rsqrtf(nn);
      float prod = 0.f;
      const int v0 = sFaceNodes[f * NF], vn = sOpp[f];
      for (int a = 0; a < D; ++a) {
        nv[a] *= nn;
        prod += (X[vn * D + a] - X[v0 * D + a]) * nv[a];
      }
      if (prod > 0.f)
        for (int a = 0; a < D; ++a) nv[a] = -nv[a];
      ds *= fw[k];
      float tq = 0.f;
      for (int i = 0; i < NF; ++i) tq += fphi[k * NF + i] * tauL[f * NF + i];
      dSt[fk] = ds * tq;
      for (int a = 0; a < D; ++a) dSn[fk * D + a] = ds * nv[a];
      for (int a = 0; a < D; ++a) {
        float acc = 0.f;
        for (int b = 0; b < D; ++b) {
          float kab = 0.f;
          for (int i = 0; i < NF; ++i) kab += fphi[k * NF + i] * kapN[sFaceNodes[f * NF + i] * D * D + a + b * D];
          acc += kab * nv[b];
        }
        dSkn[fk * D + a] = ds * acc;
      }
    }
    __syncthreads();
    // ------------------------------- volume coefficient rows -> A (hi, lo)
    {
      constexpr int KC = T::NIP / 4;
      // walk the tiles in shared-memory order (core matrices of 8 rows x 4 values), so that
      // consecutive threads store to consecutive words
      for (int o = tid; o < T::TV * 128 * T::NIP; o += kThreads) {
        const int t = o / (128 * T::NIP), oo = o % (128 * T::NIP);
        const int r = t * 128 + (oo / (KC * 32)) * 8 + (oo / 4) % 8, q = ((oo / 32) % KC) * 4 + (oo % 4);
        float v = 0.f;
        if (r < T::RV && q < NI) {
          if (r < 2 * D * N) {
            const float* Jm = (r < D * N) ? IJ : KIJ;
            const int d = (r / N) % D, i = r % N;
            for (int c = 0; c < D; ++c) v += Jm[(q * D + d) * D + c] * dphi[(q * N + i) * D + c];
          } else {
            v = dV[q] * phi[q * N + (r - 2 * D * N)];
          }
        }
        const float hi = tf32_hi(v);
        aHi[o] = hi;
        aLo[o] = tf32_hi(v - hi);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0) {
      issue_tiles(tmem, T::TV, T::NIP, T::NVB, aHiS, aLoS, tabS + T::TB_VHI * 4, tabS + T::TB_VLO * 4);
      mma_commit(&bars[1]);
    }
    // source load f_u = Phi^T (f dV) on the CUDA cores meanwhile (Source.cpp:24-48)
    for (int i = tid; i < N; i += kThreads) {
      float acc = 0.f;
      for (int q = 0; q < NI; ++q) acc += phi[q * N + i] * fq[q];
      out[T::RV * N + T::RF * NF + i] = acc;
    }
    if (!mbar_wait(&bars[1], phase)) {
      atomicCAS(p.status, 0, 2);
      sAbort = 1;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // drain: warp w holds rows 32w.. of every tile; stage them in A hi (free now) and
    // write each tile's valid rows as one contiguous run
    for (int t = 0; t < T::TV; ++t) {
      float v[32];
      tmem_ld<32>(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(t * T::NVB), v);
      const int r = 32 * warp + lane;
      constexpr int SV = N | 1;  // odd row stride: the 32 rows of a warp hit 32 banks
#pragma unroll
      for (int j = 0; j < N; ++j) aHi[r * SV + j] = v[j];
      __syncthreads();
      const int rows = (T::RV - t * 128) < 128 ? (T::RV - t * 128) : 128;
      float* dst = out + (int64_t)t * 128 * N;
      for (int i = tid; i < rows * N; i += kThreads) dst[i] = aHi[(i / N) * SV + i % N];
      __syncthreads();
    }
    // ------------------------------------ face coefficient rows -> A (hi, lo)
    {
      constexpr int KC = T::NIFP / 4;
      for (int o = tid; o < T::TF * 128 * T::NIFP; o += kThreads) {
        const int t = o / (128 * T::NIFP), oo = o % (128 * T::NIFP);
        const int r = t * 128 + (oo / (KC * 32)) * 8 + (oo / 4) % 8, k = ((oo / 32) % KC) * 4 + (oo % 4);
        float v = 0.f;
        if (r < T::RF && k < NIF) {
          if (r < F * NF) {
            const int f = r / NF, a = r % NF;
            v = dSt[f * NIF + k] * fphi[k * NF + a];
          } else {
            const int rr = (r - F * NF) % (F * D * NF);
            const float* src = (r < F * NF + F * D * NF) ? dSn : dSkn;
            const int f = rr / (D * NF), d = (rr / NF) % D, a = rr % NF;
            v = src[(f * NIF + k) * D + d] * fphi[k * NF + a];
          }
        }
        const float hi = tf32_hi(v);
        aHi[o] = hi;
        aLo[o] = tf32_hi(v - hi);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0 && !sAbort) {
      issue_tiles(tmem + (uint32_t)(T::TV * T::NVB), T::TF, T::NIFP, T::NFB, aHiS, aLoS, tabS + T::TB_FHI * 4,
                  tabS + T::TB_FLO * 4);
      mma_commit(&bars[1]);
    }
    if (!sAbort && !mbar_wait(&bars[1], phase)) {
      atomicCAS(p.status, 0, 2);
      sAbort = 1;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    for (int t = 0; t < T::TF; ++t) {
      float v[16];
      tmem_ld<16>(tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(T::TV * T::NVB + t * T::NFB), v);
      const int r = 32 * warp + lane;
      constexpr int SF = NF | 1;
#pragma unroll
      for (int j = 0; j < NF; ++j) aHi[r * SF + j] = v[j];
      __syncthreads();
      const int rows = (T::RF - t * 128) < 128 ? (T::RF - t * 128) : 128;
      float* dst = out + T::RV * N + (int64_t)t * 128 * NF;
      for (int i = tid; i < rows * NF; i += kThreads) dst[i] = aHi[(i / NF) * SF + i % NF];
      __syncthreads();
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)T::TMEM_COLS));
}

// ------------------------------------------------ CG element operators
// Mass (Mass.cpp:5-38), Diffusion (Diffusion.cpp:5-43) and Convection (Convection.cpp:21-46)
// as the same contractions: mass rows a = dV phi_i against B = phi (K = the IPs); diffusion
// rows a[(q, c)] = sum_r Gamma_q[c][r] d_r phi_i with Gamma_q = dV J^{-T} K_q J^{-1}, and
// convection rows a[(q, c)] = phi_k beta_q[c] with beta_q = dV J^{-T} v_q, both against
// B = the reference gradients (K = IPs x dimensions). Two MMA phases share the A buffer.
template <int D, int P>
struct CgTcDims {
  using K = Dims<D, P>;
  static constexpr int N = K::N, NI = K::NI;
  static constexpr int NIP = (NI + 7) / 8 * 8;
  static constexpr int KD = NI * D, KDP = (KD + 7) / 8 * 8;
  static constexpr int NB = 32;  // MMA N (nodes, padded)
  static constexpr int A_FLOATS = 128 * (KDP > NIP ? KDP : NIP);
  static constexpr int TB_PHI_HI = 0, TB_PHI_LO = TB_PHI_HI + NB * NIP;
  static constexpr int TB_DP_HI = TB_PHI_LO + NB * NIP, TB_DP_LO = TB_DP_HI + NB * KDP;
  static constexpr int TB_PHI = TB_DP_LO + NB * KDP, TB_DPHI = TB_PHI + NI * N, TB_W = TB_DPHI + NI * N * D;
  static constexpr int TB_FLOATS = (TB_W + NI + 3) / 4 * 4;
  // per-element scratch: X, dV, Gamma [NI][D][D], beta [NI][D]
  static constexpr int S_X = 0, S_DV = S_X + N * D, S_GAM = S_DV + NI, S_BETA = S_GAM + NI * D * D;
  static constexpr int S_FLOATS = (S_BETA + NI * D + 3) / 4 * 4;
  static constexpr size_t OFF_AHI = 0, OFF_ALO = (size_t)A_FLOATS * 4, OFF_TAB = OFF_ALO + (size_t)A_FLOATS * 4;
  static constexpr size_t OFF_SCR = OFF_TAB + (size_t)TB_FLOATS * 4;
  static constexpr size_t SMEM = OFF_SCR + (size_t)S_FLOATS * 4 + 1024;
  static constexpr int TMEM_COLS = 64;
};

template <int D, int P>
__global__ void __launch_bounds__(kThreads) tc_cg_operators(CgOpParams p) {
  using T = CgTcDims<D, P>;
  constexpr int N = T::N, NI = T::NI;
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  float* aHi = (float*)(smem + T::OFF_AHI);
  float* aLo = (float*)(smem + T::OFF_ALO);
  float* tab = (float*)(smem + T::OFF_TAB);
  float* scr = (float*)(smem + T::OFF_SCR);
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t tmemBase;
  __shared__ int sAbort;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[0])));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[1])));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    sAbort = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmemBase)),
                 "r"((uint32_t)T::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = tmemBase;
  if (tid == 0) {
    const uint32_t bytes = (uint32_t)T::TB_FLOATS * 4u;
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(&bars[0])), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(tab)),
                 "l"(p.tctab), "r"(bytes), "r"(smem_u32(&bars[0]))
                 : "memory");
  }
  if (!mbar_wait(&bars[0], 0)) {
    atomicCAS(p.status, 0, 2);
    sAbort = 1;
  }
  __syncthreads();
  const float* phi = tab + T::TB_PHI;
  const float* dphi = tab + T::TB_DPHI;
  const float* w = tab + T::TB_W;
  float* X = scr + T::S_X;
  float* dV = scr + T::S_DV;
  float* Gam = scr + T::S_GAM;
  float* beta = scr + T::S_BETA;
  const uint32_t aHiS = smem_u32(aHi), aLoS = smem_u32(aLo), tabS = smem_u32(tab);
  uint32_t phase = 0;
  for (int64_t e = blockIdx.x; e < p.nCells && !sAbort; e += gridDim.x) {
    const int* cell = p.cells + e * N;
    for (int i = tid; i < N * D; i += kThreads) X[i] = (float)p.coords[(int64_t)cell[i / D] * D + (i % D)];
    __syncthreads();
    for (int q = tid; q < NI; q += kThreads) {
      float J[D][D];
      for (int r = 0; r < D; ++r)
        for (int s = 0; s < D; ++s) {
          float acc = 0.f;
          for (int i = 0; i < N; ++i) acc += dphi[(q * N + i) * D + r] * X[i * D + s];
          J[r][s] = acc;
        }
      float det, iv[D][D];
      if (D == 2) {
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        const float id = 1.f / det;
        iv[0][0] = J[1][1] * id;
        iv[0][1] = -J[0][1] * id;
        iv[1][0] = -J[1][0] * id;
        iv[1][1] = J[0][0] * id;
      } else {
        const float c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const float c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const float c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        const float id = 1.f / det;
        iv[0][0] = c00 * id;
        iv[1][0] = c01 * id;
        iv[2][0] = c02 * id;
        iv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
        iv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
        iv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
        iv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
        iv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
        iv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
      }
      const float dv = w[q] * det;
      dV[q] = dv;
      float K[D][D], v[D];
      for (int a = 0; a < D; ++a) {
        for (int b = 0; b < D; ++b) {
          float acc = (p.kc == 0 && a == b) ? 1.f : 0.f;
          if (p.kc > 0)
            for (int j = 0; j < N; ++j) {
              const int64_t bk = p.kappaLayout == 0 ? (int64_t)cell[j] * p.kc : (e * N + j) * p.kc;
              const float kv = p.kc == 1 ? (a == b ? (float)p.kappa[bk] : 0.f) : (float)p.kappa[bk + a + b * D];
              acc += phi[q * N + j] * kv;
            }
          K[a][b] = acc;
        }
        float acc = 0.f;
        if (p.vel)
          for (int j = 0; j < N; ++j) {
            const int64_t bv = p.velLayout == 0 ? (int64_t)cell[j] * D : (e * N + j) * D;
            acc += phi[q * N + j] * (float)p.vel[bv + a];
          }
        v[a] = acc;
      }
      // Gamma = dV J^{-T} K J^{-1} ([c][r]), beta = dV J^{-T} v
      for (int c = 0; c < D; ++c) {
        for (int r = 0; r < D; ++r) {
          float acc = 0.f;
          for (int a = 0; a < D; ++a)
            for (int b = 0; b < D; ++b) acc += iv[a][c] * K[a][b] * iv[b][r];
          Gam[(q * D + c) * D + r] = dv * acc;
        }
        float bb = 0.f;
        for (int a = 0; a < D; ++a) bb += v[a] * iv[a][c];
        beta[q * D + c] = dv * bb;
      }
    }
    __syncthreads();
    double* out = p.out + e * 3 * N * N;
    // phase 1: mass rows against phi
    {
      constexpr int KC = T::NIP / 4;
      for (int o = tid; o < 128 * T::NIP; o += kThreads) {  // shared-memory order
        const int r = (o / (KC * 32)) * 8 + (o / 4) % 8, q = ((o / 32) % KC) * 4 + (o % 4);
        const float val = (r < N && q < NI) ? dV[q] * phi[q * N + r] : 0.f;
        const float hi = tf32_hi(val);
        aHi[o] = hi;
        aLo[o] = tf32_hi(val - hi);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0) {
      issue_tiles(tmem, 1, T::NIP, T::NB, aHiS, aLoS, tabS + T::TB_PHI_HI * 4, tabS + T::TB_PHI_LO * 4);
      mma_commit(&bars[1]);
    }
    if (!mbar_wait(&bars[1], phase)) {
      atomicCAS(p.status, 0, 2);
      sAbort = 1;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    {
      float v[32];
      tmem_ld<32>(tmem + ((uint32_t)(32 * warp) << 16), v);
      const int r = 32 * warp + lane;
      if ((p.which & 1) && r < N)
#pragma unroll
        for (int j = 0; j < N; ++j) out[j * N + r] = (double)v[j];
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // phase 2: diffusion rows then convection rows against the reference gradients
    {
      constexpr int KC = T::KDP / 4;
      for (int o = tid; o < 128 * T::KDP; o += kThreads) {  // shared-memory order
        const int r = (o / (KC * 32)) * 8 + (o / 4) % 8, k = ((o / 32) % KC) * 4 + (o % 4);
        float val = 0.f;
        if (k < T::KD && r < 2 * N) {
          const int q = k / D, c = k % D;
          if (r < N) {
            for (int s = 0; s < D; ++s) val += Gam[(q * D + c) * D + s] * dphi[(q * N + r) * D + s];
          } else {
            val = phi[q * N + (r - N)] * beta[q * D + c];
          }
        }
        const float hi = tf32_hi(val);
        aHi[o] = hi;
        aLo[o] = tf32_hi(val - hi);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (tid == 0 && !sAbort) {
      issue_tiles(tmem + 32u, 1, T::KDP, T::NB, aHiS, aLoS, tabS + T::TB_DP_HI * 4, tabS + T::TB_DP_LO * 4);
      mma_commit(&bars[1]);
    }
    if (!sAbort && !mbar_wait(&bars[1], phase)) {
      atomicCAS(p.status, 0, 2);
      sAbort = 1;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    {
      float v[32];
      tmem_ld<32>(tmem + ((uint32_t)(32 * warp) << 16) + 32u, v);
      const int r = 32 * warp + lane;
      if (r < N && (p.which & 2))
#pragma unroll
        for (int j = 0; j < N; ++j) out[N * N + j * N + r] = (double)v[j];
      if (r >= N && r < 2 * N && (p.which & 4))
#pragma unroll
        for (int j = 0; j < N; ++j) out[2 * N * N + j * N + (r - N)] = (double)v[j];
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)T::TMEM_COLS));
}

// Resident CTAs per SM for a kernel of `threads` threads and `smem` bytes of dynamic shared
// memory: the occupancy API's answer, checked against the kernel's registers and shared
// memory and the SM's 512 TMEM columns (tcols per CTA); the larger of the API's answer and
// the resource count is used (extra CTAs only queue: the CTAs do not wait on one another).
template <class K>
int resident_ctas(K kern, int threads, size_t smem, int tcols) {
  int dev = 0, perSM = 0;
  cudaGetDevice(&dev);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kern, threads, smem) != cudaSuccess) perSM = 1;
  cudaFuncAttributes a{};
  int smemSM = 0, resv = 0, regsSM = 0;
  if (cudaFuncGetAttributes(&a, kern) == cudaSuccess &&
      cudaDeviceGetAttribute(&smemSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev) == cudaSuccess &&
      cudaDeviceGetAttribute(&regsSM, cudaDevAttrMaxRegistersPerMultiprocessor, dev) == cudaSuccess) {
    const size_t perCta = smem + a.sharedSizeBytes + (size_t)resv;
    const int bySmem = perCta > 0 ? (int)((size_t)smemSM / perCta) : 1;
    const int regsCta = ((a.numRegs * 32 + 255) / 256 * 256) * ((threads + 31) / 32);
    const int byRegs = regsCta > 0 ? regsSM / regsCta : 1;
    const int calc = bySmem < byRegs ? bySmem : byRegs;
    if (calc > perSM) perSM = calc;
  }
  if (perSM * tcols > 512) perSM = 512 / tcols;
  return perSM < 1 ? 1 : perSM;
}

// ---------------------------------------------------------------- host side
double tf32_round_host(double x) {
  float f = (float)x;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u = (u + 0x1000u) & ~0x1FFFu;  // round to nearest (ties away), 10 explicit mantissa bits
  std::memcpy(&f, &u, 4);
  return (double)f;
}

template <int D, int P>
std::vector<float> build_table(const double* tab64) {
  using T = TcDims<D, P>;
  constexpr int N = T::N, NF = T::NF, NI = T::NI, NIF = T::NIF, DM = T::DM;
  const double* phi = tab64;
  const double* dphi = phi + NI * N;
  const double* w = dphi + NI * N * D;
  const double* fphi = w + NI;
  const double* fdphi = fphi + NIF * NF;
  const double* fw = fdphi + NIF * NF * DM;
  std::vector<float> t(T::TB_FLOATS, 0.f);
  // B images: row = output column (node j / face node b), K = integration point
  for (int j = 0; j < N; ++j)
    for (int q = 0; q < NI; ++q) {
      const double x = phi[q * N + j], hi = tf32_round_host(x);
      t[T::TB_VHI + cm_index(j, q, T::NIP / 4)] = (float)hi;
      t[T::TB_VLO + cm_index(j, q, T::NIP / 4)] = (float)tf32_round_host(x - hi);
    }
  for (int b = 0; b < NF; ++b)
    for (int k = 0; k < NIF; ++k) {
      const double x = fphi[k * NF + b], hi = tf32_round_host(x);
      t[T::TB_FHI + cm_index(b, k, T::NIFP / 4)] = (float)hi;
      t[T::TB_FLO + cm_index(b, k, T::NIFP / 4)] = (float)tf32_round_host(x - hi);
    }
  for (int i = 0; i < NI * N; ++i) t[T::TB_PHI + i] = (float)phi[i];
  for (int i = 0; i < NI * N * D; ++i) t[T::TB_DPHI + i] = (float)dphi[i];
  for (int i = 0; i < NI; ++i) t[T::TB_W + i] = (float)w[i];
  for (int i = 0; i < NIF * NF; ++i) t[T::TB_FPHI + i] = (float)fphi[i];
  for (int i = 0; i < NIF * NF * DM; ++i) t[T::TB_FDPHI + i] = (float)fdphi[i];
  for (int i = 0; i < NIF; ++i) t[T::TB_FW + i] = (float)fw[i];
  return t;
}

template <int D, int P>
std::vector<float> build_cg_table(const double* tab64) {
  using T = CgTcDims<D, P>;
  constexpr int N = T::N, NI = T::NI;
  const double* phi = tab64;
  const double* dphi = phi + NI * N;
  const double* w = dphi + NI * N * D;
  std::vector<float> t(T::TB_FLOATS, 0.f);
  for (int j = 0; j < N; ++j) {
    for (int q = 0; q < NI; ++q) {
      const double x = phi[q * N + j], hi = tf32_round_host(x);
      t[T::TB_PHI_HI + cm_index(j, q, T::NIP / 4)] = (float)hi;
      t[T::TB_PHI_LO + cm_index(j, q, T::NIP / 4)] = (float)tf32_round_host(x - hi);
      for (int c = 0; c < D; ++c) {
        const double y = dphi[(q * N + j) * D + c], yh = tf32_round_host(y);
        t[T::TB_DP_HI + cm_index(j, q * D + c, T::KDP / 4)] = (float)yh;
        t[T::TB_DP_LO + cm_index(j, q * D + c, T::KDP / 4)] = (float)tf32_round_host(y - yh);
      }
    }
  }
  for (int i = 0; i < NI * N; ++i) t[T::TB_PHI + i] = (float)phi[i];
  for (int i = 0; i < NI * N * D; ++i) t[T::TB_DPHI + i] = (float)dphi[i];
  for (int i = 0; i < NI; ++i) t[T::TB_W + i] = (float)w[i];
  return t;
}

template <int D, int P>
cudaError_t launch_cg_t(const CgOpParams& p, cudaStream_t s) {
  using T = CgTcDims<D, P>;
  auto kern = tc_cg_operators<D, P>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::SMEM);
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
  if (err != cudaSuccess) return err;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int perSM = resident_ctas(kern, kThreads, T::SMEM, T::TMEM_COLS);
  int64_t grid = (int64_t)nsm * perSM;
  if (grid > p.nCells) grid = p.nCells;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, kThreads, T::SMEM, s>>>(p);
  return cudaGetLastError();
}

template <int D, int P>
cudaError_t launch_t(const TcBlockParams& p, cudaStream_t s) {
  using T = TcDims<D, P>;
  auto kern = tc_element_blocks<D, P>;
  cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)T::SMEM);
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, (int)cudaSharedmemCarveoutMaxShared);
  if (err != cudaSuccess) return err;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int perSM = resident_ctas(kern, kThreads, T::SMEM, T::TMEM_COLS);
  int64_t grid = (int64_t)nsm * perSM;
  if (grid > p.nCells) grid = p.nCells;
  if (grid < 1) grid = 1;
  kern<<<(unsigned)grid, kThreads, T::SMEM, s>>>(p);
  return cudaGetLastError();
}

}  // namespace

bool tc_blocks_supported(int dim, int order) {
  return (dim == 2 && order >= 1 && order <= 5) || (dim == 3 && order >= 1 && order <= 3);
}

#define HFX_TC_DISPATCH(...)                 \
  if (dim == 2) {                             \
    switch (order) {                          \
      case 1: { constexpr int D = 2, P = 1; __VA_ARGS__; } \
      case 2: { constexpr int D = 2, P = 2; __VA_ARGS__; } \
      case 3: { constexpr int D = 2, P = 3; __VA_ARGS__; } \
      case 4: { constexpr int D = 2, P = 4; __VA_ARGS__; } \
      case 5: { constexpr int D = 2, P = 5; __VA_ARGS__; } \
    }                                         \
  } else if (dim == 3) {                      \
    switch (order) {                          \
      case 1: { constexpr int D = 3, P = 1; __VA_ARGS__; } \
      case 2: { constexpr int D = 3, P = 2; __VA_ARGS__; } \
      case 3: { constexpr int D = 3, P = 3; __VA_ARGS__; } \
    }                                         \
  }

int64_t tc_blocks_stride(int dim, int order) {
  HFX_TC_DISPATCH(return TcDims<D, P>::OUT_STRIDE);
  return 0;
}

std::vector<float> tc_table(int dim, int order, const double* tab64) {
  HFX_TC_DISPATCH(return build_table<D, P>(tab64));
  return {};
}

cudaError_t launch_tc_blocks(int dim, int order, const TcBlockParams& p, cudaStream_t s) {
  HFX_TC_DISPATCH(return launch_t<D, P>(p, s));
  return cudaErrorInvalidValue;
}

std::vector<float> tc_cg_table(int dim, int order, const double* tab64) {
  HFX_TC_DISPATCH(return build_cg_table<D, P>(tab64));
  return {};
}

cudaError_t launch_cg_operators_tc(int dim, int order, const CgOpParams& p, cudaStream_t s) {
  HFX_TC_DISPATCH(return launch_cg_t<D, P>(p, s));
  return cudaErrorInvalidValue;
}

}  // namespace hfx
