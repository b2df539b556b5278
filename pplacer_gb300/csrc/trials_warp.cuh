// Stage-2 trials, one WARP per (query, location) optimisation: the form for
// nucleotide models with Gamma rate mixtures (K = 4, RP = 1, 2, 4 or 8 rates)
// and with per-site CAT categories (sites_warp_cat).
// Included by engine.cu after trials.cuh, inside its anonymous namespace.
//
// The CTA-per-trial kernel (trials.cuh) stages the query's sites in shared
// memory and evaluates them with all the CTA's warps; between evaluations
// the optimiser step, the exp factors and the matrices are short serial
// phases that leave most warps waiting at block barriers.  Here each warp
// owns a whole trial, so those phases of one trial overlap the site loops of
// the other trials resident on the SM, and no block barrier is taken after
// the prologue.  The windows are read from global memory in every
// evaluation, streamed by cp.async into a per-warp ring of kWarpRing
// iterations, so each lane has that many site loads in flight without
// holding them in registers.
//
// Lane layout: lane = slot * RP + r.  A lane evaluates rate r of sites
// slot, slot + 32 / RP, ...; it holds rate r's six 4x4 matrices in
// registers for the whole evaluation.  The RP lanes of a site add their rate
// terms with shuffles: for 2 and 4 rates a reduce-scatter over RP
// consecutive iterations leaves each lane one whole site per group to
// accumulate; for 8 rates an all-reduce, lane r == 0 accumulating; a single
// rate needs none.  The evaluation's final xor all-reduce leaves the
// warp's sums identical in every lane, so every lane runs the same optimiser
// step; the request is still broadcast from lane 0 so control flow stays
// uniform by construction.

constexpr int kWarpTrialWarps = 1;  // warps (trials) per CTA
// Resident one-warp CTAs per SM the register allocation aims for.  A warp's
// registers come from one scheduler's file: 8 warps (2 per scheduler) leave
// 255 registers each, 12 (3 per scheduler) only 168.  With 255 the compiler
// interleaves the unrolled site iterations, which measured 6.6% faster than
// the third warp per scheduler.
constexpr int kWarpTrialMinCtas = 8;
constexpr int kWarpRing = 8;        // site iterations in flight per warp

__host__ __device__ inline size_t warp_trial_const_floats(int NM, int ncode) {
  return 16 + 64 + 2 * (size_t)ncode * 4 + 4 + (size_t)NM * 4;
}
// zc: the character codes the query-vector tables hold (c.zcodes); mats:
// the per-model transition matrices (every form but the CAT eigenbasis
// form, which holds 12 floats per category instead)
__host__ __device__ inline size_t warp_trial_table_floats(int NM, int zc, bool mats = true) {
  return (mats ? 6 * (size_t)NM * 16 : 12 * (size_t)NM) + 3 * (size_t)NM * zc * 4 + 2 * 3 * (size_t)NM * 4;
}
static_assert(kWarpRing == 8, "ring depth 8: the codes in flight fill one 64-bit register");

// The trials of one launch: the concatenation of up to 8 index lists (the
// query-length bins, longest first, so the longest trials start first);
// list[k] == nullptr stands for the identity start[k], start[k] + 1, ...
struct WarpSegs {
  const int *list[8];
  int start[9];
  int nseg, n;  // n = start[nseg]
};
// per warp: its tables, the ring of D / P float4s [2][kWarpRing][32], and
// the optimiser state
__host__ __device__ inline size_t warp_trial_warp_bytes(int NM, int zc, bool mats = true) {
  return align16(4 * warp_trial_table_floats(NM, zc, mats)) + 2 * kWarpRing * 32 * 16 + align16(sizeof(Optimiser));
}
__host__ __device__ inline size_t warp_trial_smem_bytes(int NM, int ncode, int zc, bool mats = true) {
  return align16(4 * warp_trial_const_floats(NM, ncode)) + kWarpTrialWarps * warp_trial_warp_bytes(NM, zc, mats);
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// sites of one evaluation; the lane's partial (mantissa, exponent) product
// and derivative sums accumulate into acc (lanes r == 0 only)
template <int RP, bool DER>
__device__ __forceinline__ void sites_warp(const TrialCtx &c, const TrialSmem &sm, float4 *ring, int q, int node,
                                           int Sq, int lane, SiteAcc &acc) {
  constexpr int K = 4, SPW = 32 / RP;
  const int r = lane & (RP - 1), slot = lane / RP, zc = c.zcodes;
  float md[16], mp[16], md1[DER ? 16 : 1], md2[DER ? 16 : 1], mp1[DER ? 16 : 1], mp2[DER ? 16 : 1];
#pragma unroll
  for (int t = 0; t < 16; t += 4) {
    float4 a = *reinterpret_cast<const float4 *>(sm.Md + r * 16 + t);
    float4 b = *reinterpret_cast<const float4 *>(sm.Mp + r * 16 + t);
    md[t] = a.x; md[t + 1] = a.y; md[t + 2] = a.z; md[t + 3] = a.w;
    mp[t] = b.x; mp[t + 1] = b.y; mp[t + 2] = b.z; mp[t + 3] = b.w;
    if (DER) {
      float4 c1 = *reinterpret_cast<const float4 *>(sm.Md1 + r * 16 + t);
      float4 c2 = *reinterpret_cast<const float4 *>(sm.Md2 + r * 16 + t);
      float4 e1 = *reinterpret_cast<const float4 *>(sm.Mp1 + r * 16 + t);
      float4 e2 = *reinterpret_cast<const float4 *>(sm.Mp2 + r * 16 + t);
      md1[t] = c1.x; md1[t + 1] = c1.y; md1[t + 2] = c1.z; md1[t + 3] = c1.w;
      md2[t] = c2.x; md2[t + 1] = c2.y; md2[t + 2] = c2.z; md2[t + 3] = c2.w;
      mp1[t] = e1.x; mp1[t + 1] = e1.y; mp1[t + 2] = e1.z; mp1[t + 3] = e1.w;
      mp2[t] = e2.x; mp2[t + 1] = e2.y; mp2[t + 2] = e2.z; mp2[t + 3] = e2.w;
    }
  }
  const float *gd = c.darr + (long)node * c.S * RP * K + r * K;
  const float *gp = c.parr + (long)node * c.S * RP * K + r * K;
  const uint32_t *rc = c.rcode + (long)q * c.S;
  const float *Zr = sm.Z + r * zc * K, *Z1r = sm.Z1 + r * zc * K, *Z2r = sm.Z2 + r * zc * K;
  const int last = Sq - 1;
  // Iterations come in groups of G; in iteration k of a group the lane
  // evaluates position k ^ r of the group (for 2 and 4 rates), so that the
  // reduce-scatter below needs no selects.  Site of iteration j:
  // (j / G) * G * SPW + off[j % G].
  constexpr int G = (RP == 2 || RP == 4) ? RP : 1;
  int off[G];
#pragma unroll
  for (int k = 0; k < G; k++) off[k] = (G > 1 ? (k ^ r) : 0) * SPW + slot;
  // Ring stage of iteration j: j % kWarpRing.  Iteration j issues the copy of
  // iteration j + kWarpRing - 1 into the stage iteration j - 1 consumed, and
  // loads the (column, code) word of iteration j + kWarpRing + 1, two
  // iterations before its copy is issued; the site of iteration
  // j + kWarpRing is the site of j plus kWarpRing * SPW.
  // Sites past the end read the last site and are not accumulated.  A lane
  // reads back only ring entries it copied itself, so the per-thread
  // wait_group is the only synchronisation the ring needs.  The character
  // codes of the iterations in flight travel in a register, byte k holding
  // the code of the k-th next iteration, so the evolved-query loads of an
  // iteration need no shared-memory round trip first.
  unsigned long long cq = 0ull;
  auto issue = [&](int stage, uint32_t pk) {
    const long col = (long)(pk >> 8);
    cp_async16(ring + (stage * 32 + lane), gd + col * RP * K);
    cp_async16(ring + ((kWarpRing + stage) * 32 + lane), gp + col * RP * K);
    cp_async_commit();
  };
#pragma unroll
  for (int j = 0; j < kWarpRing - 1; j++) {
    const uint32_t pk = rc[min((j / G) * G * SPW + off[j % G], last)];
    issue(j, pk);
    cq |= (unsigned long long)(pk & 255u) << (8 * j);
  }
  uint32_t pk_next = rc[min(((kWarpRing - 1) / G) * G * SPW + off[(kWarpRing - 1) % G], last)];
  uint32_t pk_next2 = rc[min(off[0] + kWarpRing * SPW, last)];
  int st = 0;
  // i: the lane's site in this iteration; inext: in the next one
  auto iteration = [&](int i, int inext, float (&v)[6]) {
    issue((st + kWarpRing - 1) & (kWarpRing - 1), pk_next);
    cq |= (unsigned long long)(pk_next & 255u) << (8 * (kWarpRing - 1));
    const int code = (int)(cq & 255ull);
    cq >>= 8;
    pk_next = pk_next2;
    pk_next2 = rc[min(inext + kWarpRing * SPW, last)];
    cp_async_wait<kWarpRing - 1>();  // this iteration's copies have landed
    const float4 dcur = ring[st * 32 + lane];
    const float4 pcur = ring[(kWarpRing + st) * 32 + lane];
    st = (st + 1) & (kWarpRing - 1);
    const float dv[4] = {dcur.x, dcur.y, dcur.z, dcur.w}, pv[4] = {pcur.x, pcur.y, pcur.z, pcur.w};
    const float4 Z4 = *reinterpret_cast<const float4 *>(Zr + code * K);
    const float z[4] = {Z4.x, Z4.y, Z4.z, Z4.w};
    float z1[4], z2[4];
    if (DER) {
      float4 a = *reinterpret_cast<const float4 *>(Z1r + code * K);
      float4 b = *reinterpret_cast<const float4 *>(Z2r + code * K);
      z1[0] = a.x; z1[1] = a.y; z1[2] = a.z; z1[3] = a.w;
      z2[0] = b.x; z2[1] = b.y; z2[2] = b.z; z2[3] = b.w;
    }
#pragma unroll
    for (int k = 0; k < 6; k++) v[k] = 0.f;
#pragma unroll
    for (int ii = 0; ii < 4; ii++) {
      float x = 0.f, y = 0.f;
#pragma unroll
      for (int jj = 0; jj < 4; jj++) {
        x = fmaf(md[ii * 4 + jj], dv[jj], x);
        y = fmaf(mp[ii * 4 + jj], pv[jj], y);
      }
      float xy = x * y;
      v[0] = fmaf(z[ii], xy, v[0]);
      if (DER) {
        float x1 = 0.f, x2 = 0.f, y1 = 0.f, y2 = 0.f;
#pragma unroll
        for (int jj = 0; jj < 4; jj++) {
          x1 = fmaf(md1[ii * 4 + jj], dv[jj], x1);
          x2 = fmaf(md2[ii * 4 + jj], dv[jj], x2);
          y1 = fmaf(mp1[ii * 4 + jj], pv[jj], y1);
          y2 = fmaf(mp2[ii * 4 + jj], pv[jj], y2);
        }
        float aa = x1 * y - x * y1;
        float bb = x2 * y - 2.f * x1 * y1 + x * y2;
        v[1] = fmaf(z[ii], aa, v[1]);
        v[2] = fmaf(z[ii], bb, v[2]);
        v[3] = fmaf(z1[ii], xy, v[3]);
        v[4] = fmaf(z2[ii], xy, v[4]);
        v[5] = fmaf(z1[ii], aa, v[5]);
      }
    }
  };
  constexpr int NV = DER ? 6 : 1;
  for (int gbase = 0; gbase < Sq; gbase += G * SPW) {
    float f[6];
    if (G == 4) {
      // v_k holds position k ^ r.  Stage xor 1: the partner's v1 (v3) is at
      // the position of this lane's v0 (v2); stage xor 2: the partner's h1
      // is at this lane's position r.
      float v0[6], v1[6], h0[6], h1[6];
      iteration(gbase + off[0], gbase + off[1], v0);
      iteration(gbase + off[1], gbase + off[2], v1);
#pragma unroll
      for (int k = 0; k < NV; k++) h0[k] = v0[k] + __shfl_xor_sync(0xffffffffu, v1[k], 1);
      iteration(gbase + off[2], gbase + off[3], v0);
      iteration(gbase + off[3], gbase + G * SPW + off[0], v1);
#pragma unroll
      for (int k = 0; k < NV; k++) h1[k] = v0[k] + __shfl_xor_sync(0xffffffffu, v1[k], 1);
#pragma unroll
      for (int k = 0; k < NV; k++) f[k] = h0[k] + __shfl_xor_sync(0xffffffffu, h1[k], 2);
    } else if (G == 2) {
      float v0[6], v1[6];
      iteration(gbase + off[0], gbase + off[1], v0);
      iteration(gbase + off[1], gbase + G * SPW + off[0], v1);
#pragma unroll
      for (int k = 0; k < NV; k++) f[k] = v0[k] + __shfl_xor_sync(0xffffffffu, v1[k], 1);
    } else {
      // one rate: the lane's own site; eight rates: xor all-reduce
      iteration(gbase + off[0], gbase + SPW + off[0], f);
#pragma unroll
      for (int o = 1; o < RP; o <<= 1)
#pragma unroll
        for (int k = 0; k < NV; k++) f[k] += __shfl_xor_sync(0xffffffffu, f[k], o);
    }
    const bool mine = G > 1 ? gbase + r * SPW + slot < Sq : (r == 0 && gbase + slot < Sq);
    if (mine) acc.add(f[0], f[1], f[2], f[3], f[4], f[5], DER);
  }
  cp_async_wait<0>();  // drain the copies issued past the end
}

// Eigen-coordinates of the nucleotide windows for sites_warp_eig: rows
// (node, site, rate) of darr and parr times X^-1 (FP64 accumulation), slot 0
// the zero eigenvalue's coordinate times its constant eigenvector entry c0,
// slots 1..3 the other coordinates in eig_ord order.
__global__ void k_eigen_glvs_dna(const float *__restrict__ darr, const float *__restrict__ parr,
                                 const double *__restrict__ Xit, long rows, int eig_ord, double c0, float *darr_e,
                                 float *parr_e) {
  constexpr int K = 4;
  int ord[4];
#pragma unroll
  for (int k = 0; k < 4; k++) ord[k] = (eig_ord >> (8 * k)) & 255;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < 2 * rows; t += (long)gridDim.x * blockDim.x) {
    const bool prox = t >= rows;
    const long row = prox ? t - rows : t;
    const float *v = (prox ? parr : darr) + row * K;
    float *o = (prox ? parr_e : darr_e) + row * K;
    float x[K];
#pragma unroll
    for (int j = 0; j < K; j++) x[j] = v[j];
#pragma unroll
    for (int s = 0; s < K; s++) {
      const int k = ord[s];
      double a = 0.0;
#pragma unroll
      for (int j = 0; j < K; j++) a += Xit[j * K + k] * (double)x[j];  // (X^-1)[k][j] = Xit[j][k]
      o[s] = (float)(s == 0 ? c0 * a : a);
    }
  }
}

// The same sites in the eigenbasis of the rate matrix (the autotuner's
// second warp form for nucleotide Gamma mixtures).  With P(t) = X diag(e^{r
// lambda t}) X^-1 and the windows stored as eigen-coordinates v~ = X^-1 v
// (k_eigen_glvs_dna), x = P(t) d is X (e o d~), and its first and second
// length derivatives are X (r lambda e o d~) and X ((r lambda)^2 e o d~).
// The zero eigenvalue's eigenvector is constant, so its term is the same for
// every state: the arrays store it premultiplied in slot 0 and the other
// three eigen-coordinates in slots 1..3 (the order c.eig_ord).  A lane then
// holds X's three other columns, the same scaled by r lambda and (r
// lambda)^2, and three exp factors per window instead of six 4x4 matrices
// (42 registers instead of 96); a new branch length only changes the
// factors, and the arithmetic per site and rate drops from 96 to 78 FMA-pipe
// operations for the six evolved vectors (3 scalings of the coordinates per
// window, then 12 FMA per vector).
template <int RP, bool DER>
__device__ __forceinline__ void sites_warp_eig(const TrialCtx &c, const TrialSmem &sm, float4 *ring, int q, int node,
                                               int Sq, int lane, SiteAcc &acc) {
  constexpr int K = 4, SPW = 32 / RP;
  const int r = lane & (RP - 1), slot = lane / RP, zc = c.zcodes, NM = c.NM;
  int ord[3];
  ord[0] = (c.eig_ord >> 8) & 255; ord[1] = (c.eig_ord >> 16) & 255; ord[2] = (c.eig_ord >> 24) & 255;
  // xl1, xl2: the columns scaled by r lambda and (r lambda)^2, so the
  // derivative vectors come from the same scaled coordinates e o d~
  float xr[4][3], xl1[4][3], xl2[4][3], ed[3], ep[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float lr = sm.Lr[r * K + ord[k]];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      xr[i][k] = sm.X[i * K + ord[k]];
      xl1[i][k] = xr[i][k] * lr;
      xl2[i][k] = xl1[i][k] * lr;
    }
    ed[k] = sm.E[(0 * NM + r) * K + ord[k]];
    ep[k] = sm.E[(1 * NM + r) * K + ord[k]];
  }
  const float *gd = c.darr_e + (long)node * c.S * RP * K + r * K;
  const float *gp = c.parr_e + (long)node * c.S * RP * K + r * K;
  const uint32_t *rc = c.rcode + (long)q * c.S;
  const float *Zr = sm.Z + r * zc * K, *Z1r = sm.Z1 + r * zc * K, *Z2r = sm.Z2 + r * zc * K;
  const int last = Sq - 1;
  constexpr int G = (RP == 2 || RP == 4) ? RP : 1;
  int off[G];
#pragma unroll
  for (int k = 0; k < G; k++) off[k] = (G > 1 ? (k ^ r) : 0) * SPW + slot;
  // the ring, the code queue and the iteration order are those of sites_warp
  unsigned long long cq = 0ull;
  auto issue = [&](int stage, uint32_t pk) {
    const long col = (long)(pk >> 8);
    cp_async16(ring + (stage * 32 + lane), gd + col * RP * K);
    cp_async16(ring + ((kWarpRing + stage) * 32 + lane), gp + col * RP * K);
    cp_async_commit();
  };
#pragma unroll
  for (int j = 0; j < kWarpRing - 1; j++) {
    const uint32_t pk = rc[min((j / G) * G * SPW + off[j % G], last)];
    issue(j, pk);
    cq |= (unsigned long long)(pk & 255u) << (8 * j);
  }
  uint32_t pk_next = rc[min(((kWarpRing - 1) / G) * G * SPW + off[(kWarpRing - 1) % G], last)];
  uint32_t pk_next2 = rc[min(off[0] + kWarpRing * SPW, last)];
  int st = 0;
  auto iteration = [&](int i, int inext, float (&v)[6]) {
    issue((st + kWarpRing - 1) & (kWarpRing - 1), pk_next);
    cq |= (unsigned long long)(pk_next & 255u) << (8 * (kWarpRing - 1));
    const int code = (int)(cq & 255ull);
    cq >>= 8;
    pk_next = pk_next2;
    pk_next2 = rc[min(inext + kWarpRing * SPW, last)];
    cp_async_wait<kWarpRing - 1>();  // this iteration's copies have landed
    const float4 dcur = ring[st * 32 + lane];
    const float4 pcur = ring[(kWarpRing + st) * 32 + lane];
    st = (st + 1) & (kWarpRing - 1);
    const float dv[3] = {dcur.y, dcur.z, dcur.w}, pv[3] = {pcur.y, pcur.z, pcur.w};
    const float4 Z4 = *reinterpret_cast<const float4 *>(Zr + code * K);
    const float z[4] = {Z4.x, Z4.y, Z4.z, Z4.w};
    float z1[4], z2[4];
    if (DER) {
      float4 a = *reinterpret_cast<const float4 *>(Z1r + code * K);
      float4 b = *reinterpret_cast<const float4 *>(Z2r + code * K);
      z1[0] = a.x; z1[1] = a.y; z1[2] = a.z; z1[3] = a.w;
      z2[0] = b.x; z2[1] = b.y; z2[2] = b.z; z2[3] = b.w;
    }
    float ud[3], wp[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      ud[k] = ed[k] * dv[k];
      wp[k] = ep[k] * pv[k];
    }
#pragma unroll
    for (int k = 0; k < 6; k++) v[k] = 0.f;
#pragma unroll
    for (int ii = 0; ii < 4; ii++) {
      float x = dcur.x, y = pcur.x;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        x = fmaf(xr[ii][k], ud[k], x);
        y = fmaf(xr[ii][k], wp[k], y);
      }
      float xy = x * y;
      v[0] = fmaf(z[ii], xy, v[0]);
      if (DER) {
        float x1 = xl1[ii][0] * ud[0], x2 = xl2[ii][0] * ud[0], y1 = xl1[ii][0] * wp[0], y2 = xl2[ii][0] * wp[0];
#pragma unroll
        for (int k = 1; k < 3; k++) {
          x1 = fmaf(xl1[ii][k], ud[k], x1);
          x2 = fmaf(xl2[ii][k], ud[k], x2);
          y1 = fmaf(xl1[ii][k], wp[k], y1);
          y2 = fmaf(xl2[ii][k], wp[k], y2);
        }
        float aa = x1 * y - x * y1;
        float bb = x2 * y - 2.f * x1 * y1 + x * y2;
        v[1] = fmaf(z[ii], aa, v[1]);
        v[2] = fmaf(z[ii], bb, v[2]);
        v[3] = fmaf(z1[ii], xy, v[3]);
        v[4] = fmaf(z2[ii], xy, v[4]);
        v[5] = fmaf(z1[ii], aa, v[5]);
      }
    }
  };
  constexpr int NV = DER ? 6 : 1;
  for (int gbase = 0; gbase < Sq; gbase += G * SPW) {
    float f[6];
    if (G == 4) {
      float v0[6], v1[6], h0[6], h1[6];
      iteration(gbase + off[0], gbase + off[1], v0);
      iteration(gbase + off[1], gbase + off[2], v1);
#pragma unroll
      for (int k = 0; k < NV; k++) h0[k] = v0[k] + __shfl_xor_sync(0xffffffffu, v1[k], 1);
      iteration(gbase + off[2], gbase + off[3], v0);
      iteration(gbase + off[3], gbase + G * SPW + off[0], v1);
#pragma unroll
      for (int k = 0; k < NV; k++) h1[k] = v0[k] + __shfl_xor_sync(0xffffffffu, v1[k], 1);
#pragma unroll
      for (int k = 0; k < NV; k++) f[k] = h0[k] + __shfl_xor_sync(0xffffffffu, h1[k], 2);
    } else if (G == 2) {
      float v0[6], v1[6];
      iteration(gbase + off[0], gbase + off[1], v0);
      iteration(gbase + off[1], gbase + G * SPW + off[0], v1);
#pragma unroll
      for (int k = 0; k < NV; k++) f[k] = v0[k] + __shfl_xor_sync(0xffffffffu, v1[k], 1);
    } else {
      iteration(gbase + off[0], gbase + SPW + off[0], f);
#pragma unroll
      for (int o = 1; o < RP; o <<= 1)
#pragma unroll
        for (int k = 0; k < NV; k++) f[k] += __shfl_xor_sync(0xffffffffu, f[k], o);
    }
    const bool mine = G > 1 ? gbase + r * SPW + slot < Sq : (r == 0 && gbase + slot < Sq);
    if (mine) acc.add(f[0], f[1], f[2], f[3], f[4], f[5], DER);
  }
  cp_async_wait<0>();  // drain the copies issued past the end
}

// The eigenbasis form on packed FP32 pairs (fma.rn.f32x2, two lanes of
// arithmetic per instruction): the states (0, 1) and (2, 3) of a site share
// each instruction -- X's columns pair across the two states, the scaled
// eigen-coordinates are duplicated into both halves -- so the evolves and
// the six sums take about 74 instructions per site and rate instead of 130.
// The proximal first derivative is formed negated (-y') with the negated
// exp factors, as it only enters the sums as -x y' and -2 x' y'.
template <int RP, bool DER>
__device__ __forceinline__ void sites_warp_eig2(const TrialCtx &c, const TrialSmem &sm, float4 *ring, int q, int node,
                                                int Sq, int lane, SiteAcc &acc) {
  constexpr int K = 4, SPW = 32 / RP;
  const int r = lane & (RP - 1), slot = lane / RP, zc = c.zcodes, NM = c.NM;
  int ord[3];
  ord[0] = (c.eig_ord >> 8) & 255; ord[1] = (c.eig_ord >> 16) & 255; ord[2] = (c.eig_ord >> 24) & 255;
  // xp[h][k] = (X[2h][k], X[2h+1][k]); xq1, xq2 the same scaled by r lambda, (r lambda)^2
  float2 xp[2][3], xq1[2][3], xq2[2][3];
  float ed[3], ep[3], epn[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float lr = sm.Lr[r * K + ord[k]];
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const float a = sm.X[(2 * h) * K + ord[k]], b = sm.X[(2 * h + 1) * K + ord[k]];
      const float a1 = a * lr, b1 = b * lr;
      xp[h][k] = make_float2(a, b);
      xq1[h][k] = make_float2(a1, b1);
      xq2[h][k] = make_float2(a1 * lr, b1 * lr);
    }
    ed[k] = sm.E[(0 * NM + r) * K + ord[k]];
    ep[k] = sm.E[(1 * NM + r) * K + ord[k]];
    epn[k] = -ep[k];
  }
  const float *gd = c.darr_e + (long)node * c.S * RP * K + r * K;
  const float *gp = c.parr_e + (long)node * c.S * RP * K + r * K;
  const uint32_t *rc = c.rcode + (long)q * c.S;
  const float *Zr = sm.Z + r * zc * K, *Z1r = sm.Z1 + r * zc * K, *Z2r = sm.Z2 + r * zc * K;
  const int last = Sq - 1;
  constexpr int G = (RP == 2 || RP == 4) ? RP : 1;
  int off[G];
#pragma unroll
  for (int k = 0; k < G; k++) off[k] = (G > 1 ? (k ^ r) : 0) * SPW + slot;
  // the ring, the code queue and the iteration order are those of sites_warp
  unsigned long long cq = 0ull;
  auto issue = [&](int stage, uint32_t pk) {
    const long col = (long)(pk >> 8);
    cp_async16(ring + (stage * 32 + lane), gd + col * RP * K);
    cp_async16(ring + ((kWarpRing + stage) * 32 + lane), gp + col * RP * K);
    cp_async_commit();
  };
#pragma unroll
  for (int j = 0; j < kWarpRing - 1; j++) {
    const uint32_t pk = rc[min((j / G) * G * SPW + off[j % G], last)];
    issue(j, pk);
    cq |= (unsigned long long)(pk & 255u) << (8 * j);
  }
  uint32_t pk_next = rc[min(((kWarpRing - 1) / G) * G * SPW + off[(kWarpRing - 1) % G], last)];
  uint32_t pk_next2 = rc[min(off[0] + kWarpRing * SPW, last)];
  int st = 0;
  auto iteration = [&](int i, int inext, float (&v)[6]) {
    issue((st + kWarpRing - 1) & (kWarpRing - 1), pk_next);
    cq |= (unsigned long long)(pk_next & 255u) << (8 * (kWarpRing - 1));
    const int code = (int)(cq & 255ull);
    cq >>= 8;
    pk_next = pk_next2;
    pk_next2 = rc[min(inext + kWarpRing * SPW, last)];
    cp_async_wait<kWarpRing - 1>();  // this iteration's copies have landed
    const float4 dcur = ring[st * 32 + lane];
    const float4 pcur = ring[(kWarpRing + st) * 32 + lane];
    st = (st + 1) & (kWarpRing - 1);
    const float dv[3] = {dcur.y, dcur.z, dcur.w}, pv[3] = {pcur.y, pcur.z, pcur.w};
    const float4 Z4 = *reinterpret_cast<const float4 *>(Zr + code * K);
    const float2 zz[2] = {make_float2(Z4.x, Z4.y), make_float2(Z4.z, Z4.w)};
    float2 z1p[2], z2p[2];
    if (DER) {
      const float4 a = *reinterpret_cast<const float4 *>(Z1r + code * K);
      const float4 b = *reinterpret_cast<const float4 *>(Z2r + code * K);
      z1p[0] = make_float2(a.x, a.y); z1p[1] = make_float2(a.z, a.w);
      z2p[0] = make_float2(b.x, b.y); z2p[1] = make_float2(b.z, b.w);
    }
    float2 ud[3], wp[3], wn[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float u = ed[k] * dv[k], w = ep[k] * pv[k];
      ud[k] = make_float2(u, u);
      wp[k] = make_float2(w, w);
      if (DER) {
        const float wq = epn[k] * pv[k];
        wn[k] = make_float2(wq, wq);
      }
    }
    float2 V[6];
#pragma unroll
    for (int k = 0; k < 6; k++) V[k] = make_float2(0.f, 0.f);
#pragma unroll
    for (int h = 0; h < 2; h++) {
      float2 X = make_float2(dcur.x, dcur.x), Y = make_float2(pcur.x, pcur.x);
#pragma unroll
      for (int k = 0; k < 3; k++) {
        X = __ffma2_rn(xp[h][k], ud[k], X);
        Y = __ffma2_rn(xp[h][k], wp[k], Y);
      }
      const float2 XY = __fmul2_rn(X, Y);
      V[0] = __ffma2_rn(zz[h], XY, V[0]);
      if (DER) {
        float2 X1 = __fmul2_rn(xq1[h][0], ud[0]), X2 = __fmul2_rn(xq2[h][0], ud[0]);
        float2 Y1n = __fmul2_rn(xq1[h][0], wn[0]), Y2 = __fmul2_rn(xq2[h][0], wp[0]);
#pragma unroll
        for (int k = 1; k < 3; k++) {
          X1 = __ffma2_rn(xq1[h][k], ud[k], X1);
          X2 = __ffma2_rn(xq2[h][k], ud[k], X2);
          Y1n = __ffma2_rn(xq1[h][k], wn[k], Y1n);
          Y2 = __ffma2_rn(xq2[h][k], wp[k], Y2);
        }
        const float2 AA = __ffma2_rn(X, Y1n, __fmul2_rn(X1, Y));                        // x' y - x y'
        const float2 BB = __ffma2_rn(X, Y2, __ffma2_rn(X1, __fadd2_rn(Y1n, Y1n), __fmul2_rn(X2, Y)));
        V[1] = __ffma2_rn(zz[h], AA, V[1]);
        V[2] = __ffma2_rn(zz[h], BB, V[2]);
        V[3] = __ffma2_rn(z1p[h], XY, V[3]);
        V[4] = __ffma2_rn(z2p[h], XY, V[4]);
        V[5] = __ffma2_rn(z1p[h], AA, V[5]);
      }
    }
#pragma unroll
    for (int k = 0; k < 6; k++) v[k] = V[k].x + V[k].y;
  };
  constexpr int NV = DER ? 6 : 1;
  for (int gbase = 0; gbase < Sq; gbase += G * SPW) {
    float f[6];
    if (G == 4) {
      float v0[6], v1[6], h0[6], h1[6];
      iteration(gbase + off[0], gbase + off[1], v0);
      iteration(gbase + off[1], gbase + off[2], v1);
#pragma unroll
      for (int k = 0; k < NV; k++) h0[k] = v0[k] + __shfl_xor_sync(0xffffffffu, v1[k], 1);
      iteration(gbase + off[2], gbase + off[3], v0);
      iteration(gbase + off[3], gbase + G * SPW + off[0], v1);
#pragma unroll
      for (int k = 0; k < NV; k++) h1[k] = v0[k] + __shfl_xor_sync(0xffffffffu, v1[k], 1);
#pragma unroll
      for (int k = 0; k < NV; k++) f[k] = h0[k] + __shfl_xor_sync(0xffffffffu, h1[k], 2);
    } else if (G == 2) {
      float v0[6], v1[6];
      iteration(gbase + off[0], gbase + off[1], v0);
      iteration(gbase + off[1], gbase + G * SPW + off[0], v1);
#pragma unroll
      for (int k = 0; k < NV; k++) f[k] = v0[k] + __shfl_xor_sync(0xffffffffu, v1[k], 1);
    } else {
      iteration(gbase + off[0], gbase + SPW + off[0], f);
#pragma unroll
      for (int o = 1; o < RP; o <<= 1)
#pragma unroll
        for (int k = 0; k < NV; k++) f[k] += __shfl_xor_sync(0xffffffffu, f[k], o);
    }
    const bool mine = G > 1 ? gbase + r * SPW + slot < Sq : (r == 0 && gbase + slot < Sq);
    if (mine) acc.add(f[0], f[1], f[2], f[3], f[4], f[5], DER);
  }
  cp_async_wait<0>();  // drain the copies issued past the end
}

// Sites of a per-site CAT model (Gcat_model, one GLV plane): lane = site,
// 32 sites per iteration, the windows streamed through the same cp.async
// ring.  A site's matrices are those of its category (the packed word's top
// byte) and are read from the shared tables in every iteration: a query's
// sites come grouped by category (k_query_prep), so the lanes of an
// iteration mostly read one category's matrices as a broadcast.
template <bool DER>
__device__ __forceinline__ void sites_warp_cat(const TrialCtx &c, const TrialSmem &sm, float4 *ring, int q, int node,
                                               int Sq, int lane, SiteAcc &acc) {
  constexpr int K = 4;
  const int zc = c.zcodes;
  const float *gd = c.darr + (long)node * c.S * K;
  const float *gp = c.parr + (long)node * c.S * K;
  const uint32_t *rc = c.rcode + (long)q * c.S;
  const int last = Sq - 1;
  // byte k of cq / kq: the character / category of the k-th next iteration
  unsigned long long cq = 0ull, kq = 0ull;
  auto issue = [&](int stage, uint32_t pk) {
    const long col = (long)((pk >> 8) & 0xffffu);
    cp_async16(ring + (stage * 32 + lane), gd + col * K);
    cp_async16(ring + ((kWarpRing + stage) * 32 + lane), gp + col * K);
    cp_async_commit();
  };
#pragma unroll
  for (int j = 0; j < kWarpRing - 1; j++) {
    const uint32_t pk = rc[min(j * 32 + lane, last)];
    issue(j, pk);
    cq |= (unsigned long long)(pk & 255u) << (8 * j);
    kq |= (unsigned long long)(pk >> 24) << (8 * j);
  }
  uint32_t pk_next = rc[min((kWarpRing - 1) * 32 + lane, last)];
  uint32_t pk_next2 = rc[min(kWarpRing * 32 + lane, last)];
  int st = 0;
  for (int base = 0; base < Sq; base += 32) {
    issue((st + kWarpRing - 1) & (kWarpRing - 1), pk_next);
    cq |= (unsigned long long)(pk_next & 255u) << (8 * (kWarpRing - 1));
    kq |= (unsigned long long)(pk_next >> 24) << (8 * (kWarpRing - 1));
    const int code = (int)(cq & 255ull), cat = (int)(kq & 255ull);
    cq >>= 8;
    kq >>= 8;
    pk_next = pk_next2;
    pk_next2 = rc[min(base + 32 + kWarpRing * 32 + lane, last)];
    cp_async_wait<kWarpRing - 1>();  // this iteration's copies have landed
    const float4 dcur = ring[st * 32 + lane];
    const float4 pcur = ring[(kWarpRing + st) * 32 + lane];
    st = (st + 1) & (kWarpRing - 1);
    const float dv[4] = {dcur.x, dcur.y, dcur.z, dcur.w}, pv[4] = {pcur.x, pcur.y, pcur.z, pcur.w};
    const float *Md = sm.Md + cat * 16, *Mp = sm.Mp + cat * 16;
    const float4 Z4 = *reinterpret_cast<const float4 *>(sm.Z + (cat * zc + code) * K);
    const float z[4] = {Z4.x, Z4.y, Z4.z, Z4.w};
    float z1[4], z2[4];
    if (DER) {
      const float4 a = *reinterpret_cast<const float4 *>(sm.Z1 + (cat * zc + code) * K);
      const float4 b = *reinterpret_cast<const float4 *>(sm.Z2 + (cat * zc + code) * K);
      z1[0] = a.x; z1[1] = a.y; z1[2] = a.z; z1[3] = a.w;
      z2[0] = b.x; z2[1] = b.y; z2[2] = b.z; z2[3] = b.w;
    }
    float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int ii = 0; ii < 4; ii++) {
      const float4 a = *reinterpret_cast<const float4 *>(Md + ii * 4);
      const float4 b = *reinterpret_cast<const float4 *>(Mp + ii * 4);
      const float x = a.x * dv[0] + a.y * dv[1] + a.z * dv[2] + a.w * dv[3];
      const float y = b.x * pv[0] + b.y * pv[1] + b.z * pv[2] + b.w * pv[3];
      const float xy = x * y;
      v[0] = fmaf(z[ii], xy, v[0]);
      if (DER) {
        const float4 a1 = *reinterpret_cast<const float4 *>(sm.Md1 + cat * 16 + ii * 4);
        const float4 a2 = *reinterpret_cast<const float4 *>(sm.Md2 + cat * 16 + ii * 4);
        const float4 b1 = *reinterpret_cast<const float4 *>(sm.Mp1 + cat * 16 + ii * 4);
        const float4 b2 = *reinterpret_cast<const float4 *>(sm.Mp2 + cat * 16 + ii * 4);
        const float x1 = a1.x * dv[0] + a1.y * dv[1] + a1.z * dv[2] + a1.w * dv[3];
        const float x2 = a2.x * dv[0] + a2.y * dv[1] + a2.z * dv[2] + a2.w * dv[3];
        const float y1 = b1.x * pv[0] + b1.y * pv[1] + b1.z * pv[2] + b1.w * pv[3];
        const float y2 = b2.x * pv[0] + b2.y * pv[1] + b2.z * pv[2] + b2.w * pv[3];
        const float aa = x1 * y - x * y1;
        const float bb = x2 * y - 2.f * x1 * y1 + x * y2;
        v[1] = fmaf(z[ii], aa, v[1]);
        v[2] = fmaf(z[ii], bb, v[2]);
        v[3] = fmaf(z1[ii], xy, v[3]);
        v[4] = fmaf(z2[ii], xy, v[4]);
        v[5] = fmaf(z1[ii], aa, v[5]);
      }
    }
    if (base + lane < Sq) acc.add(v[0], v[1], v[2], v[3], v[4], v[5], DER);
  }
  cp_async_wait<0>();  // drain the copies issued past the end
}

// The CAT model in the eigenbasis: every category shares the rate matrix's
// eigenvectors, so the windows are stored as eigen-coordinates (one plane,
// the layout of k_eigen_glvs_dna) and a site's category enters only through
// three exp factors per window and three r lambda scalings, read from the
// warp's 12-float table of the category (Tc: exp(r lambda_k dist),
// exp(r lambda_k prox), r lambda_k for the three non-zero eigenvalues in
// eig_ord order) -- 3 shared loads per site instead of the 24 of six 4x4
// matrices, and tables small enough for more warps per SM.
__device__ __forceinline__ void cat_eig_tables(const TrialCtx &c, const TrialSmem &sm, int NM, int lane) {
  constexpr int K = 4;
  const int o1 = (c.eig_ord >> 8) & 255, o2 = (c.eig_ord >> 16) & 255, o3 = (c.eig_ord >> 24) & 255;
  for (int it = lane; it < 12 * NM; it += 32) {
    const int cat = it / 12, j = it - cat * 12, g = j / 3, kk = j - g * 3;
    const int o = kk == 0 ? o1 : (kk == 1 ? o2 : o3);
    sm.Tc[it] = g == 0 ? sm.E[cat * K + o] : (g == 1 ? sm.E[(NM + cat) * K + o] : (g == 2 ? sm.Lr[cat * K + o] : 0.f));
  }
}

template <bool DER>
__device__ __forceinline__ void sites_warp_cat_eig(const TrialCtx &c, const TrialSmem &sm, float4 *ring, int q,
                                                   int node, int Sq, int lane, SiteAcc &acc) {
  constexpr int K = 4;
  const int zc = c.zcodes;
  int ord[3];
  ord[0] = (c.eig_ord >> 8) & 255; ord[1] = (c.eig_ord >> 16) & 255; ord[2] = (c.eig_ord >> 24) & 255;
  float xr[4][3];
#pragma unroll
  for (int k = 0; k < 3; k++)
#pragma unroll
    for (int i = 0; i < 4; i++) xr[i][k] = sm.X[i * K + ord[k]];
  const float *gd = c.darr_e + (long)node * c.S * K;
  const float *gp = c.parr_e + (long)node * c.S * K;
  const uint32_t *rc = c.rcode + (long)q * c.S;
  const int last = Sq - 1;
  // byte k of cq / kq: the character / category of the k-th next iteration
  unsigned long long cq = 0ull, kq = 0ull;
  auto issue = [&](int stage, uint32_t pk) {
    const long col = (long)((pk >> 8) & 0xffffu);
    cp_async16(ring + (stage * 32 + lane), gd + col * K);
    cp_async16(ring + ((kWarpRing + stage) * 32 + lane), gp + col * K);
    cp_async_commit();
  };
#pragma unroll
  for (int j = 0; j < kWarpRing - 1; j++) {
    const uint32_t pk = rc[min(j * 32 + lane, last)];
    issue(j, pk);
    cq |= (unsigned long long)(pk & 255u) << (8 * j);
    kq |= (unsigned long long)(pk >> 24) << (8 * j);
  }
  uint32_t pk_next = rc[min((kWarpRing - 1) * 32 + lane, last)];
  uint32_t pk_next2 = rc[min(kWarpRing * 32 + lane, last)];
  int st = 0;
  for (int base = 0; base < Sq; base += 32) {
    issue((st + kWarpRing - 1) & (kWarpRing - 1), pk_next);
    cq |= (unsigned long long)(pk_next & 255u) << (8 * (kWarpRing - 1));
    kq |= (unsigned long long)(pk_next >> 24) << (8 * (kWarpRing - 1));
    const int code = (int)(cq & 255ull), cat = (int)(kq & 255ull);
    cq >>= 8;
    kq >>= 8;
    pk_next = pk_next2;
    pk_next2 = rc[min(base + 32 + kWarpRing * 32 + lane, last)];
    cp_async_wait<kWarpRing - 1>();  // this iteration's copies have landed
    const float4 dcur = ring[st * 32 + lane];
    const float4 pcur = ring[(kWarpRing + st) * 32 + lane];
    st = (st + 1) & (kWarpRing - 1);
    const float4 t0 = *reinterpret_cast<const float4 *>(sm.Tc + cat * 12);
    const float4 t1 = *reinterpret_cast<const float4 *>(sm.Tc + cat * 12 + 4);
    const float ed[3] = {t0.x, t0.y, t0.z}, ep[3] = {t0.w, t1.x, t1.y};
    const float4 Z4 = *reinterpret_cast<const float4 *>(sm.Z + (cat * zc + code) * K);
    const float z[4] = {Z4.x, Z4.y, Z4.z, Z4.w};
    float z1[4], z2[4], lr[3];
    if (DER) {
      const float4 t2 = *reinterpret_cast<const float4 *>(sm.Tc + cat * 12 + 8);
      lr[0] = t1.z; lr[1] = t1.w; lr[2] = t2.x;
      const float4 a = *reinterpret_cast<const float4 *>(sm.Z1 + (cat * zc + code) * K);
      const float4 b = *reinterpret_cast<const float4 *>(sm.Z2 + (cat * zc + code) * K);
      z1[0] = a.x; z1[1] = a.y; z1[2] = a.z; z1[3] = a.w;
      z2[0] = b.x; z2[1] = b.y; z2[2] = b.z; z2[3] = b.w;
    }
    const float dv[3] = {dcur.y, dcur.z, dcur.w}, pv[3] = {pcur.y, pcur.z, pcur.w};
    float ud[3], wp[3], ud1[3], ud2[3], wp1[3], wp2[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      ud[k] = ed[k] * dv[k];
      wp[k] = ep[k] * pv[k];
      if (DER) {
        ud1[k] = lr[k] * ud[k];
        ud2[k] = lr[k] * ud1[k];
        wp1[k] = lr[k] * wp[k];
        wp2[k] = lr[k] * wp1[k];
      }
    }
    float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int ii = 0; ii < 4; ii++) {
      float x = dcur.x, y = pcur.x;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        x = fmaf(xr[ii][k], ud[k], x);
        y = fmaf(xr[ii][k], wp[k], y);
      }
      const float xy = x * y;
      v[0] = fmaf(z[ii], xy, v[0]);
      if (DER) {
        float x1 = xr[ii][0] * ud1[0], x2 = xr[ii][0] * ud2[0], y1 = xr[ii][0] * wp1[0], y2 = xr[ii][0] * wp2[0];
#pragma unroll
        for (int k = 1; k < 3; k++) {
          x1 = fmaf(xr[ii][k], ud1[k], x1);
          x2 = fmaf(xr[ii][k], ud2[k], x2);
          y1 = fmaf(xr[ii][k], wp1[k], y1);
          y2 = fmaf(xr[ii][k], wp2[k], y2);
        }
        const float aa = x1 * y - x * y1;
        const float bb = x2 * y - 2.f * x1 * y1 + x * y2;
        v[1] = fmaf(z[ii], aa, v[1]);
        v[2] = fmaf(z[ii], bb, v[2]);
        v[3] = fmaf(z1[ii], xy, v[3]);
        v[4] = fmaf(z2[ii], xy, v[4]);
        v[5] = fmaf(z1[ii], aa, v[5]);
      }
    }
    if (base + lane < Sq) acc.add(v[0], v[1], v[2], v[3], v[4], v[5], DER);
  }
  cp_async_wait<0>();  // drain the copies issued past the end
}

// The CAT eigenbasis form on packed FP32 pairs: the arithmetic of
// sites_warp_cat_eig with two states of the site per fma.rn.f32x2 (X's
// columns paired across the states, the site's scaled eigen-coordinates
// duplicated into both halves, the proximal first derivative formed
// negated as in sites_warp_eig2).
template <bool DER>
__device__ __forceinline__ void sites_warp_cat_eig2(const TrialCtx &c, const TrialSmem &sm, float4 *ring, int q,
                                                    int node, int Sq, int lane, SiteAcc &acc) {
  constexpr int K = 4;
  const int zc = c.zcodes;
  int ord[3];
  ord[0] = (c.eig_ord >> 8) & 255; ord[1] = (c.eig_ord >> 16) & 255; ord[2] = (c.eig_ord >> 24) & 255;
  float2 xp[2][3];
#pragma unroll
  for (int k = 0; k < 3; k++)
#pragma unroll
    for (int h = 0; h < 2; h++) xp[h][k] = make_float2(sm.X[(2 * h) * K + ord[k]], sm.X[(2 * h + 1) * K + ord[k]]);
  const float *gd = c.darr_e + (long)node * c.S * K;
  const float *gp = c.parr_e + (long)node * c.S * K;
  const uint32_t *rc = c.rcode + (long)q * c.S;
  const int last = Sq - 1;
  unsigned long long cq = 0ull, kq = 0ull;
  auto issue = [&](int stage, uint32_t pk) {
    const long col = (long)((pk >> 8) & 0xffffu);
    cp_async16(ring + (stage * 32 + lane), gd + col * K);
    cp_async16(ring + ((kWarpRing + stage) * 32 + lane), gp + col * K);
    cp_async_commit();
  };
#pragma unroll
  for (int j = 0; j < kWarpRing - 1; j++) {
    const uint32_t pk = rc[min(j * 32 + lane, last)];
    issue(j, pk);
    cq |= (unsigned long long)(pk & 255u) << (8 * j);
    kq |= (unsigned long long)(pk >> 24) << (8 * j);
  }
  uint32_t pk_next = rc[min((kWarpRing - 1) * 32 + lane, last)];
  uint32_t pk_next2 = rc[min(kWarpRing * 32 + lane, last)];
  int st = 0;
  for (int base = 0; base < Sq; base += 32) {
    issue((st + kWarpRing - 1) & (kWarpRing - 1), pk_next);
    cq |= (unsigned long long)(pk_next & 255u) << (8 * (kWarpRing - 1));
    kq |= (unsigned long long)(pk_next >> 24) << (8 * (kWarpRing - 1));
    const int code = (int)(cq & 255ull), cat = (int)(kq & 255ull);
    cq >>= 8;
    kq >>= 8;
    pk_next = pk_next2;
    pk_next2 = rc[min(base + 32 + kWarpRing * 32 + lane, last)];
    cp_async_wait<kWarpRing - 1>();  // this iteration's copies have landed
    const float4 dcur = ring[st * 32 + lane];
    const float4 pcur = ring[(kWarpRing + st) * 32 + lane];
    st = (st + 1) & (kWarpRing - 1);
    const float4 t0 = *reinterpret_cast<const float4 *>(sm.Tc + cat * 12);
    const float4 t1 = *reinterpret_cast<const float4 *>(sm.Tc + cat * 12 + 4);
    const float ed[3] = {t0.x, t0.y, t0.z}, ep[3] = {t0.w, t1.x, t1.y};
    const float4 Z4 = *reinterpret_cast<const float4 *>(sm.Z + (cat * zc + code) * K);
    const float2 zz[2] = {make_float2(Z4.x, Z4.y), make_float2(Z4.z, Z4.w)};
    float2 z1p[2], z2p[2];
    float lr[3];
    if (DER) {
      const float4 t2 = *reinterpret_cast<const float4 *>(sm.Tc + cat * 12 + 8);
      lr[0] = t1.z; lr[1] = t1.w; lr[2] = t2.x;
      const float4 a = *reinterpret_cast<const float4 *>(sm.Z1 + (cat * zc + code) * K);
      const float4 b = *reinterpret_cast<const float4 *>(sm.Z2 + (cat * zc + code) * K);
      z1p[0] = make_float2(a.x, a.y); z1p[1] = make_float2(a.z, a.w);
      z2p[0] = make_float2(b.x, b.y); z2p[1] = make_float2(b.z, b.w);
    }
    const float dv[3] = {dcur.y, dcur.z, dcur.w}, pv[3] = {pcur.y, pcur.z, pcur.w};
    float2 ud[3], wp[3], ud1[3], ud2[3], wn1[3], wp2[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const float u = ed[k] * dv[k], w = ep[k] * pv[k];
      ud[k] = make_float2(u, u);
      wp[k] = make_float2(w, w);
      if (DER) {
        const float u1 = lr[k] * u, w1 = lr[k] * w;
        const float u2 = lr[k] * u1, w2 = lr[k] * w1;
        ud1[k] = make_float2(u1, u1);
        ud2[k] = make_float2(u2, u2);
        wn1[k] = make_float2(-w1, -w1);
        wp2[k] = make_float2(w2, w2);
      }
    }
    float2 V[6];
#pragma unroll
    for (int k = 0; k < 6; k++) V[k] = make_float2(0.f, 0.f);
#pragma unroll
    for (int h = 0; h < 2; h++) {
      float2 X = make_float2(dcur.x, dcur.x), Y = make_float2(pcur.x, pcur.x);
#pragma unroll
      for (int k = 0; k < 3; k++) {
        X = __ffma2_rn(xp[h][k], ud[k], X);
        Y = __ffma2_rn(xp[h][k], wp[k], Y);
      }
      const float2 XY = __fmul2_rn(X, Y);
      V[0] = __ffma2_rn(zz[h], XY, V[0]);
      if (DER) {
        float2 X1 = __fmul2_rn(xp[h][0], ud1[0]), X2 = __fmul2_rn(xp[h][0], ud2[0]);
        float2 Y1n = __fmul2_rn(xp[h][0], wn1[0]), Y2 = __fmul2_rn(xp[h][0], wp2[0]);
#pragma unroll
        for (int k = 1; k < 3; k++) {
          X1 = __ffma2_rn(xp[h][k], ud1[k], X1);
          X2 = __ffma2_rn(xp[h][k], ud2[k], X2);
          Y1n = __ffma2_rn(xp[h][k], wn1[k], Y1n);
          Y2 = __ffma2_rn(xp[h][k], wp2[k], Y2);
        }
        const float2 AA = __ffma2_rn(X, Y1n, __fmul2_rn(X1, Y));
        const float2 BB = __ffma2_rn(X, Y2, __ffma2_rn(X1, __fadd2_rn(Y1n, Y1n), __fmul2_rn(X2, Y)));
        V[1] = __ffma2_rn(zz[h], AA, V[1]);
        V[2] = __ffma2_rn(zz[h], BB, V[2]);
        V[3] = __ffma2_rn(z1p[h], XY, V[3]);
        V[4] = __ffma2_rn(z2p[h], XY, V[4]);
        V[5] = __ffma2_rn(z1p[h], AA, V[5]);
      }
    }
    if (base + lane < Sq)
      acc.add(V[0].x + V[0].y, V[1].x + V[1].y, V[2].x + V[2].y, V[3].x + V[3].y, V[4].x + V[4].y,
              V[5].x + V[5].y, DER);
  }
  cp_async_wait<0>();  // drain the copies issued past the end
}

// Per-CTA constants and this warp's tables and ring; returns after a block
// barrier, the only one the warp kernels take.
__device__ __forceinline__ void warp_trial_setup(const TrialCtx &c, char *t_smem, TrialSmem &sm, float4 *&ring,
                                                 bool mats = true) {
  constexpr int K = 4;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int NM = c.NM, nc = c.ncode;
  float *cst = reinterpret_cast<float *>(t_smem);
  sm = TrialSmem{};
  sm.X = cst;
  sm.W = cst + 16;
  sm.Lt = cst + 80;
  sm.lv = sm.Lt + nc * K;
  sm.statd = sm.lv + nc * K;
  sm.Lr = sm.statd + 4;
  for (int i = tid; i < 16; i += blockDim.x) sm.X[i] = c.X[i];
  for (int i = tid; i < 64; i += blockDim.x) sm.W[i] = c.W[i];
  for (int i = tid; i < nc * K; i += blockDim.x) { sm.Lt[i] = c.Lt[i]; sm.lv[i] = c.lvf[i]; }
  for (int i = tid; i < NM * K; i += blockDim.x) sm.Lr[i] = c.rates[i / K] * c.lam[i % K];
  if (tid < K) sm.statd[tid] = c.statd[tid];
  const int zc = c.zcodes;
  char *wb = t_smem + align16(4 * warp_trial_const_floats(NM, nc)) + warp * warp_trial_warp_bytes(NM, zc, mats);
  float *tb = reinterpret_cast<float *>(wb);
  ring = reinterpret_cast<float4 *>(wb + align16(4 * warp_trial_table_floats(NM, zc, mats)));
  sm.opt = wb + align16(4 * warp_trial_table_floats(NM, zc, mats)) + 2 * kWarpRing * 32 * 16;
  const int mb = NM * 16, zb = NM * zc * K;
  if (mats) {
    sm.Md = tb; sm.Mp = tb + mb; sm.Md1 = tb + 2 * mb; sm.Md2 = tb + 3 * mb; sm.Mp1 = tb + 4 * mb;
    sm.Mp2 = tb + 5 * mb;
    sm.Z = tb + 6 * mb;
  } else {
    sm.Tc = tb;
    sm.Z = tb + 12 * NM;
  }
  sm.Z1 = sm.Z + zb; sm.Z2 = sm.Z1 + zb;
  sm.E = sm.Z2 + zb; sm.Em1 = sm.E + 3 * NM * K;
  __syncthreads();
}

// One trial (Three_tax.optimize at one location) by the calling warp.  Every
// lane runs the same optimiser on the same all-reduced values and returns
// the same result.
template <int RP, bool CAT = false, int EIG = 0>
__device__ TrialRes trial_warp(const TrialCtx &c, const TrialSmem &sm, float4 *ring, int lane, const TrialIn &tr) {
  constexpr int K = 4;
  const int NM = c.NM, nc = c.ncode;
  const int q = tr.q, node = tr.node;
  const int Sq = c.qlen[q];
  const int ncz = c.qamb[q] > 0 ? nc : c.prim;  // Z rows the query's codes use
  // exponent sum of the query's sites of darr / parr[node]
  // (sixteen unconditional gathers in flight per lane: past the end they
  // read the last site and add nothing)
  long long esum = 0;
  {
    const long qo = (long)q * c.S, nb = (long)node * c.S;
    const int last = Sq - 1;
    for (int i0 = lane; i0 < Sq; i0 += 16 * 32) {
      int col[16];
#pragma unroll
      for (int k = 0; k < 16; k++) col[k] = c.reind[qo + min(i0 + 32 * k, last)];
      int part = 0;
#pragma unroll
      for (int k = 0; k < 16; k++) {
        const int v = c.dexp[nb + col[k]] + c.pexp[nb + col[k]];
        part += i0 + 32 * k < Sq ? v : 0;
      }
      esum += part;
    }
  }
  for (int o = 16; o > 0; o >>= 1) esum += __shfl_xor_sync(0xffffffffu, esum, o);

  // The optimiser state lives in shared memory, one copy per warp, and only
  // lane 0 runs it; the other lanes receive each request by shuffle.
  Optimiser &opt = *static_cast<Optimiser *>(sm.opt);
  if (lane == 0) {
    opt.optimizer = c.optimizer;
    opt.mode = c.mode;
    opt.cut = c.bl[node];
    opt.tol = tr.tol;
    opt.max_pend = c.max_pend;
    opt.start_pend = c.start_pend;
    opt.pend0 = tr.pend0;
    opt.dist0 = tr.dist0;
    opt.cst = kLn2 * (double)esum - (double)(float)Sq * c.log_nrates;
    opt.n_evals = 0;
    opt.seeded = tr.seeded != 0;
    opt.seed = tr.seed;
    if (tr.marginal) opt.mode = 2;
    opt.prior_kind = tr.prior_kind;
    opt.pp_rule = c.pp_rule;
    opt.pp_rel = c.pp_rel_err;
    opt.prior_mu = tr.prior_mu;
    opt.gl = c.gl;
    opt.pc = 0;
    opt.L_last = NAN;
    opt.last.ex = 0; opt.last.lm = 0.f;
    opt.last.g[0] = opt.last.g[1] = opt.last.h[0] = opt.last.h[1] = opt.last.h[2] = 0.f;
  }
  EvalOut res;
  for (int ev = 0; ev < kMaxTrialEvals; ev++) {
    int cmd = 0;
    float rp = 0.f, rd = 0.f, rx = 0.f;
    if (lane == 0) {
      bool more = opt.next(ev == 0 ? nullptr : &res);
      cmd = more ? (opt.req_derivs ? 2 : 1) : 0;
      rp = opt.req_p; rd = opt.req_d; rx = opt.req_x;
    }
    Ctrl ctl;
    ctl.cmd = __shfl_sync(0xffffffffu, cmd, 0);
    if (ctl.cmd == 0) break;
    ctl.pend = __shfl_sync(0xffffffffu, rp, 0);
    ctl.dist = __shfl_sync(0xffffffffu, rd, 0);
    ctl.prox = __shfl_sync(0xffffffffu, rx, 0);
    const bool derivs = ctl.cmd == 2;
    __syncwarp();  // the previous evaluation's sites have read the tables
    trial_exps(sm, NM, K, ctl, lane, 32);
    __syncwarp();
    trial_tables(sm, sm.W, NM, c.zcodes, ncz, K, derivs, lane, 32, !EIG);  // Z rows of stride zcodes
    if (CAT && EIG) cat_eig_tables(c, sm, NM, lane);
    __syncwarp();
    SiteAcc acc;
    acc.init();
    if (Sq > 0) {
      if (CAT && EIG == 2) {
        if (derivs) sites_warp_cat_eig2<true>(c, sm, ring, q, node, Sq, lane, acc);
        else sites_warp_cat_eig2<false>(c, sm, ring, q, node, Sq, lane, acc);
      } else if (CAT && EIG) {
        if (derivs) sites_warp_cat_eig<true>(c, sm, ring, q, node, Sq, lane, acc);
        else sites_warp_cat_eig<false>(c, sm, ring, q, node, Sq, lane, acc);
      } else if (CAT) {
        if (derivs) sites_warp_cat<true>(c, sm, ring, q, node, Sq, lane, acc);
        else sites_warp_cat<false>(c, sm, ring, q, node, Sq, lane, acc);
      } else if (EIG == 2) {
        if (derivs) sites_warp_eig2<RP, true>(c, sm, ring, q, node, Sq, lane, acc);
        else sites_warp_eig2<RP, false>(c, sm, ring, q, node, Sq, lane, acc);
      } else if (EIG) {
        if (derivs) sites_warp_eig<RP, true>(c, sm, ring, q, node, Sq, lane, acc);
        else sites_warp_eig<RP, false>(c, sm, ring, q, node, Sq, lane, acc);
      } else {
        if (derivs) sites_warp<RP, true>(c, sm, ring, q, node, Sq, lane, acc);
        else sites_warp<RP, false>(c, sm, ring, q, node, Sq, lane, acc);
      }
    }
    // xor all-reduce: every lane ends with the same bits
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      float mo = __shfl_xor_sync(0xffffffffu, acc.m, o);
      int eo = __shfl_xor_sync(0xffffffffu, acc.e, o);
      acc.m *= mo;
      acc.e += eo;
      int em;
      acc.m = frexpf(acc.m, &em);
      acc.e += em;
      if (derivs) {
        acc.gp += __shfl_xor_sync(0xffffffffu, acc.gp, o);
        acc.gd += __shfl_xor_sync(0xffffffffu, acc.gd, o);
        acc.hpp += __shfl_xor_sync(0xffffffffu, acc.hpp, o);
        acc.hdd += __shfl_xor_sync(0xffffffffu, acc.hdd, o);
        acc.hpd += __shfl_xor_sync(0xffffffffu, acc.hpd, o);
      }
    }
    res.ex = acc.e;
    res.lm = logf(acc.m);
    res.g[0] = acc.gp; res.g[1] = acc.gd;
    res.h[0] = acc.hpp; res.h[1] = acc.hdd; res.h[2] = acc.hpd;
  }
  __syncwarp();  // lane 0's final optimiser state is visible to the warp
  TrialRes rr;
  rr.like = opt.L_last;
  rr.pend = opt.pend;
  rr.dist = opt.dist;
  rr.der[0] = opt.last.g[0]; rr.der[1] = opt.last.g[1];
  rr.der[2] = opt.last.h[0]; rr.der[3] = opt.last.h[1]; rr.der[4] = opt.last.h[2];
  rr.der[5] = 0;
  rr.status = opt.status;
  rr.last = opt.last;
  rr.n_evals = opt.n_evals;
  __syncwarp();  // every lane has read the state before the next trial resets it
  if (lane == 0 && c.stats) {
    atomicAdd(&c.stats[0], (unsigned long long)opt.n_evals);
    atomicAdd(&c.stats[1], (unsigned long long)opt.n_evals * (unsigned long long)Sq);
  }
  return rr;
}

// A batch of independent trials, one per warp.
template <int RP, bool CAT = false>
__global__ void __launch_bounds__(32 * kWarpTrialWarps, kWarpTrialMinCtas)
    k_trials_warp(TrialCtx c, const TrialIn *__restrict__ trials, WarpSegs segs, TrialRes *out) {
  extern __shared__ __align__(16) char t_smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  TrialSmem sm;
  float4 *ring;
  warp_trial_setup(c, t_smem, sm, ring);
  const int t = blockIdx.x * kWarpTrialWarps + warp;
  if (t >= segs.n) return;
  // segment of t (constant indices keep segs in the parameter bank)
  const int *lst = segs.list[0];
  int s0 = 0;
#pragma unroll
  for (int k = 1; k < 8; k++)
    if (k < segs.nseg && t >= segs.start[k]) { lst = segs.list[k]; s0 = segs.start[k]; }
  const int ti = lst ? lst[t - s0] : t - s0;
  const TrialRes rr = trial_warp<RP, CAT>(c, sm, ring, lane, trials[ti]);
  if (lane == 0) out[ti] = rr;
}
