// Fused grouped sparse Compton weight on thread-block clusters (included by sparse_ops.cu).
//
// The grouped weight (recon_osem_plane_sparse.py:22-57 and the materialise form of
// recon_osem_local_sparse_jsccsd_only.py:13-19, see sparse_group_coef_bulk_kernel) in ONE
// kernel: per group g (events sharing the first-hit sysmat row A_g)
//   b_g = adj(A_g . x)          f_i = t_i . b_g          c_i = coefficient of f_i
//   q_g = sum_i c_i t_i         w  += A_g . up(q_g)
// Each byte of the event rows and of the group's sysmat row is read from HBM once, and q never
// leaves the chip (the separate kernels write b and q and read every sysmat row a second time).
//
// Data split: a cluster of kCfCluster CTAs (one per SM) works on the same groups; CTA r owns
// the rings [R0, R1) of the polar grid (one z plane, the stride-4 ring stencil: coarse voxel
// th of a ring has the fine taps 4 th + d, d = -3..3, with the polar projector's linear
// weights 1 - |d| / 4, periodic in the ring), so its fine voxels [J0, J1) and coarse voxels
// [C0, C1) close under adj and up. Every CTA stages its slice of x once, and per group its
// slice of A_g and of each event row (bulk copies of the 16-byte-aligned windows [jw0, jw1)
// and [cw0, cw1) around the slices). The only cross-CTA step is f_i = sum over the cluster
// of the CTAs' partial dots: each team's lead thread arms its own exchange mbarrier for the
// batch and writes its partials into the same exchange slot of every CTA of the cluster with
// st.async (distributed shared memory; each store completes 16 transaction bytes on the
// receiving CTA's mbarrier, so no fence is needed); partials are added in CTA order, so every
// CTA derives the same f_i and coefficient. An exchange slot is reused every kCfNX = 4
// batches, always by the same team (teams alternate batches): before a CTA writes batch b + 4
// into a peer's slot it has received that peer's partials of batch b + 2, which the peer's
// lead thread sent after reading batch b from the slot, so no slot is overwritten unread.
//
// Warp roles (512 threads, one CTA per SM):
//   warp 15       producer: bulk copies of the A_g slices (three buffers) and of the event row
//                 slices (a ring of slots), each issued as soon as its buffer is free;
//   warps 8-14    group warps: b_g for the slice into one of two buffers, then the scatter of
//                 the previous group, w_j += A_g[j] up(q_g)[j], into a partial image held in
//                 registers (kCfRuns runs of four fine voxels per thread);
//   warps 0-7     two teams of four event warps taking alternate batches of up to kCfNB
//                 events, so one team computes while the other waits for its exchange: dots
//                 (four partial sums per event), the exchange, coefficients, q in registers;
//                 at the end of a group each team stores its q into a buffer of its own, and
//                 the scatter adds the two (team 0 first).
// Every wait is bounded (g_bk_poll_limit): a CTA that gives up raises its abort flag, its
// roles leave their loops, its peers give up on their exchange waits, and every CTA waits
// (bounded) for its own copies in flight, arrives at the closing cluster barrier and counts
// the give-up (jscc_take_wait_timeout_count). Partial images: one per cluster, summed in
// cluster order by sparse_reduce_kernel. No float atomics.

constexpr int kCfCluster = 4;
constexpr int kCfThreads = 512;
constexpr int kCfTeamWarps = 4;
constexpr int kCfTeam = kCfTeamWarps * 32;  // threads per event team
constexpr int kCfGroupWarps = 7;
constexpr int kCfGroup = kCfGroupWarps * 32;
constexpr int kCfProducerWarp = 15;
constexpr int kCfNB = 4;       // events per batch
constexpr int kCfQ = 5;        // chunks of four coarse voxels per team thread (window <= 2,560)
constexpr int kCfRuns = 12;    // runs of four fine voxels per group thread (slice <= 10,752)
constexpr int kCfNX = 4;       // exchange slots
constexpr int kCfMaxSlots = 16;
constexpr int kCfHeader = 4096;
constexpr int kCfMaxWindowC = kCfTeam * 4 * kCfQ;
constexpr int kCfMaxSliceF = kCfGroup * kCfRuns * 4;
static_assert(kCfProducerWarp * 32 + 32 == kCfThreads && 2 * kCfTeam + kCfGroup + 32 == kCfThreads, "roles");

// header layout (bytes)
constexpr int kCfOffFull = 0;                       // [kCfMaxSlots] u64
constexpr int kCfOffEmpty = 128;                    // [kCfMaxSlots]
constexpr int kCfOffErowFull = 256;                 // [3]
constexpr int kCfOffErowEmpty = 280;                // [3]
constexpr int kCfOffBFull = 304;                    // [2]
constexpr int kCfOffBEmpty = 320;                   // [2]
constexpr int kCfOffQFull = 336;                    // [2]
constexpr int kCfOffQEmpty = 352;                   // [2]
constexpr int kCfOffXFull = 368;                    // [kCfNX]
constexpr int kCfOffFlags = 512;                    // abort
constexpr int kCfOffSlotIssued = 576;               // [kCfMaxSlots] int
constexpr int kCfOffSlotWaited = 640;               // [kCfMaxSlots] int
constexpr int kCfOffErowIssued = 704;               // [3] int
constexpr int kCfOffErowWaited = 720;               // [3] int
constexpr int kCfOffRed = 1024;                     // [2][kCfTeamWarps][kCfNB] float
constexpr int kCfOffCs = 1280;                      // [2][kCfNB] float
constexpr int kCfOffXval = 1536;                    // [kCfNX][kCfCluster][kCfNB] float
static_assert(kCfOffXFull + 8 * kCfNX <= kCfOffFlags, "barriers");
static_assert(kCfNX == 4, "slot reuse argument: two alternating teams, four slots");
static_assert(kCfOffXval + 4 * kCfNX * kCfCluster * kCfNB <= kCfHeader, "header");

struct CfArgs {
  const __nv_bfloat16* tc;  // split coarse rows [E, ld]
  int64_t ld;
  int64_t n_det;
  const int32_t* order;
  const int32_t* goff;
  const int32_t* grow;
  int n_groups;
  const __nv_bfloat16* eff;
  int64_t ld_eff;
  const float* x;      // fine image (already rotated)
  const float* s_ev;   // event sums by position in `order` (materialise form)
  float* part;         // [clusters][ldp] partial images
  int64_t ldp;
  int vf, vc, ring_len, n_rings;
  int n_slots;
  uint32_t x_off, erow_off, erow_stride, b_off, b_stride, q_off, q_stride, slot_off, slot_stride;
  int max_wf, max_wc;  // largest window lengths (elements) over the cluster's CTAs
};

// slice of CTA r: rings [R0, R1), fine [J0, J1), coarse [C0, C1), 16-byte windows
struct CfSlice {
  int J0, J1, C0, C1, jw0, jw1, cw0, cw1;
};
__host__ __device__ inline CfSlice cf_slice(int r, int n_rings, int ring_len, int vf, int vc) {
  CfSlice s;
  const int R0 = (int)((int64_t)n_rings * r / kCfCluster), R1 = (int)((int64_t)n_rings * (r + 1) / kCfCluster);
  const int nthc = ring_len / 4;
  s.J0 = R0 * ring_len;
  s.J1 = R1 * ring_len;
  s.C0 = R0 * nthc;
  s.C1 = R1 * nthc;
  s.jw0 = s.J0 & ~7;
  s.jw1 = ((s.J1 + 7) & ~7) < vf ? ((s.J1 + 7) & ~7) : vf;
  s.cw0 = s.C0 & ~7;
  s.cw1 = ((s.C1 + 7) & ~7) < vc ? ((s.C1 + 7) & ~7) : vc;
  return s;
}

template <int MODE>
__global__ void __launch_bounds__(kCfThreads, 1) sparse_cluster_fused_kernel(CfArgs a) {
  extern __shared__ __align__(1024) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kCfOffFull);
  uint64_t* empty = reinterpret_cast<uint64_t*>(smem + kCfOffEmpty);
  uint64_t* erow_full = reinterpret_cast<uint64_t*>(smem + kCfOffErowFull);
  uint64_t* erow_empty = reinterpret_cast<uint64_t*>(smem + kCfOffErowEmpty);
  uint64_t* b_full = reinterpret_cast<uint64_t*>(smem + kCfOffBFull);
  uint64_t* b_empty = reinterpret_cast<uint64_t*>(smem + kCfOffBEmpty);
  uint64_t* q_full = reinterpret_cast<uint64_t*>(smem + kCfOffQFull);
  uint64_t* q_empty = reinterpret_cast<uint64_t*>(smem + kCfOffQEmpty);
  uint64_t* xfull = reinterpret_cast<uint64_t*>(smem + kCfOffXFull);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + kCfOffFlags);
  int* slot_issued = reinterpret_cast<int*>(smem + kCfOffSlotIssued);
  int* slot_waited = reinterpret_cast<int*>(smem + kCfOffSlotWaited);
  int* erow_issued = reinterpret_cast<int*>(smem + kCfOffErowIssued);
  int* erow_waited = reinterpret_cast<int*>(smem + kCfOffErowWaited);
  float* red = reinterpret_cast<float*>(smem + kCfOffRed);
  float* cs = reinterpret_cast<float*>(smem + kCfOffCs);
  float* xval = reinterpret_cast<float*>(smem + kCfOffXval);
  float* xs = reinterpret_cast<float*>(smem + a.x_off);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t polls = g_bk_poll_limit;
  const uint32_t rank = cluster_rank();
  const int G = (int)n_clusters_x(), cid = (int)cluster_id_x();
  const CfSlice sl = cf_slice((int)rank, a.n_rings, a.ring_len, a.vf, a.vc);
  const int nthc = a.ring_len / 4;
  const uint32_t erow_bytes = (uint32_t)(sl.jw1 - sl.jw0) * 2u, row_bytes = (uint32_t)(sl.cw1 - sl.cw0) * 2u;
  auto erow = [&](int k) { return reinterpret_cast<__nv_bfloat16*>(smem + a.erow_off + (size_t)k * a.erow_stride); };
  auto bbuf = [&](int k) { return reinterpret_cast<float*>(smem + a.b_off + (size_t)k * a.b_stride); };
  // q buffers: [group parity][event team]
  auto qbuf = [&](int k, int team) {
    return reinterpret_cast<float*>(smem + a.q_off + (size_t)(2 * k + team) * a.q_stride);
  };
  auto slot = [&](int s) { return reinterpret_cast<__nv_bfloat16*>(smem + a.slot_off + (size_t)s * a.slot_stride); };
  if (tid == 0) {
    for (int s = 0; s < kCfMaxSlots; ++s) {
      mbar_init(full + s, 1);
      mbar_init(empty + s, 1);
      slot_issued[s] = slot_waited[s] = 0;
    }
    for (int k = 0; k < 3; ++k) {
      mbar_init(erow_full + k, 1);
      mbar_init(erow_empty + k, 1);
      erow_issued[k] = erow_waited[k] = 0;
    }
    for (int k = 0; k < 2; ++k) {
      mbar_init(b_full + k, 1);
      mbar_init(b_empty + k, 2);  // one arrival per event team
      mbar_init(q_full + k, 2);   // one arrival per event team
      mbar_init(q_empty + k, 1);
    }
    for (int k = 0; k < kCfNX; ++k) mbar_init(xfull + k, 1);  // the local arm; the peers' bytes complete it
    *abort_flag = 0;
    mbar_init_fence();
  }
  // the image slice, once: xs[j - jw0] = x[j]
  for (int j = sl.jw0 + tid; j < sl.jw1; j += kCfThreads) xs[j - sl.jw0] = __ldg(a.x + j);
  __syncthreads();
  cluster_sync_all();  // every CTA's barriers exist before any remote arrival
  const int n_mine = cid < a.n_groups ? (a.n_groups - 1 - cid) / G + 1 : 0;  // groups of this cluster

  if (warp == kCfProducerWarp) {
    // ------------------------------------------------------------ producer
    int ek = 0;                        // next group whose A_g slice is issued
    int rk = 0, re = 0, re_end = 0;    // group and event position of the next row
    if (n_mine > 0) {
      re = a.goff[cid];
      re_end = a.goff[cid + 1];
    }
    int seq = 0;
    uint32_t idle = 0;
    bool ok = true;
    while (ok) {
      while (rk < n_mine && re >= re_end) {
        ++rk;
        if (rk < n_mine) {
          const int gi = cid + rk * G;
          re = a.goff[gi];
          re_end = a.goff[gi + 1];
        }
      }
      const bool rows_left = rk < n_mine, erows_left = ek < n_mine;
      if (!rows_left && !erows_left) break;
      bool progress = false;
      if (erows_left) {
        const int k3 = ek % 3;
        bool ready = ek < 3 || mbar_test_wait(erow_empty + k3, (uint32_t)((ek / 3) - 1) & 1u);
        ready = __shfl_sync(0xffffffffu, ready, 0);
        if (ready) {
          if (lane == 0) {
            const int gi = cid + ek * G;
            const __nv_bfloat16* src = a.eff + clamp_row(a.grow[gi], a.n_det) * a.ld_eff + sl.jw0;
            mbar_arrive_expect_tx(erow_full + k3, erow_bytes);
            bulk_copy_g2s(erow(k3), src, erow_bytes, erow_full + k3);
            erow_issued[k3] += 1;
          }
          ++ek;
          progress = true;
        }
      }
      if (rows_left) {
        const int s = seq % a.n_slots;
        bool ready = seq < a.n_slots || mbar_test_wait(empty + s, (uint32_t)((seq / a.n_slots) - 1) & 1u);
        ready = __shfl_sync(0xffffffffu, ready, 0);
        if (ready) {
          if (lane == 0) {
            const int i = a.order[re];
            mbar_arrive_expect_tx(full + s, row_bytes);
            bulk_copy_g2s(slot(s), a.tc + (int64_t)i * a.ld + sl.cw0, row_bytes, full + s);
            slot_issued[s] += 1;
          }
          ++seq;
          ++re;
          progress = true;
        }
      }
      if (progress) {
        idle = 0;
      } else if (++idle > polls || *abort_flag) {
        ok = false;
      } else {
        __nanosleep(64);
      }
    }
    if (!ok && lane == 0) *abort_flag = 1;
  } else if (warp >= 2 * kCfTeamWarps) {
    // ------------------------------------------------------------ group warps
    const int gt = tid - 2 * kCfTeam;
    // the partial image of this CTA's slice in registers: runs of four fine voxels (one
    // coarse theta step of a ring: the same two coarse taps), run rho = gt + m * kCfGroup
    float acc[kCfRuns][4];
#pragma unroll
    for (int m = 0; m < kCfRuns; ++m)
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[m][i] = 0.f;
    const int n_runs = (sl.J1 - sl.J0) / 4;
    // run gt: theta index and the coarse index of theta 0 of its ring
    int th0 = gt, cb0 = sl.C0;
    while (th0 >= nthc) {
      th0 -= nthc;
      cb0 += nthc;
    }
    // this thread's first coarse voxel c = cw0 + gt: ring-relative theta and ring start
    int ath0 = sl.cw0 + gt - sl.C0, ar0 = sl.C0 / nthc;
    while (ath0 >= nthc) {
      ath0 -= nthc;
      ++ar0;
    }
    while (ath0 < 0) {
      ath0 += nthc;
      --ar0;
    }
    bool bad = false, aborted = false;
    // scatter of group k: for each run, w[4th + i] += A[4th + i] ((1 - i/4) q[th] + (i/4) q[th + 1])
    auto scatter = [&](int k) {
      if (!bk_wait(q_full + (k & 1), (uint32_t)(k >> 1) & 1u, abort_flag, polls)) bad = true;
      const __nv_bfloat16* er = erow(k % 3);
      const float* q0 = qbuf(k & 1, 0);
      const float* q1 = qbuf(k & 1, 1);
      int th = th0, cb = cb0;
#pragma unroll
      for (int m = 0; m < kCfRuns; ++m) {
        const int rho = gt + m * kCfGroup;
        if (rho < n_runs) {
          const int clo = cb + th, chi = cb + (th + 1 == nthc ? 0 : th + 1);
          const float ql = q0[clo - sl.cw0] + q1[clo - sl.cw0], qh = q0[chi - sl.cw0] + q1[chi - sl.cw0];
          const uint2 ar = *reinterpret_cast<const uint2*>(er + (sl.J0 + 4 * rho - sl.jw0));
          const float up[4] = {ql, fmaf(0.25f, qh, 0.75f * ql), fmaf(0.5f, qh, 0.5f * ql),
                               fmaf(0.75f, qh, 0.25f * ql)};
          acc[m][0] = fmaf(bf16_lo(ar.x), up[0], acc[m][0]);
          acc[m][1] = fmaf(bf16_hi(ar.x), up[1], acc[m][1]);
          acc[m][2] = fmaf(bf16_lo(ar.y), up[2], acc[m][2]);
          acc[m][3] = fmaf(bf16_hi(ar.y), up[3], acc[m][3]);
        }
        th += kCfGroup;
        while (th >= nthc) {
          th -= nthc;
          cb += nthc;
        }
      }
      if (role_sync_or(5, kCfGroup, bad)) return false;
      if (gt == 0) {
        mbar_arrive(q_empty + (k & 1));
        mbar_arrive(erow_empty + (k % 3));
      }
      return true;
    };
    // taps of the stride-4 ring stencil, d = -3..3 at positions 4 th - 4 + i, i = 1..7
    constexpr float kW[8] = {0.f, 0.25f, 0.5f, 0.75f, 1.0f, 0.75f, 0.5f, 0.25f};
    for (int kg = 0; kg < n_mine; ++kg) {
      const int k3 = kg % 3;
      if (!bk_wait(erow_full + k3, (uint32_t)(kg / 3) & 1u, abort_flag, polls)) bad = true;
      else if (gt == 0) erow_waited[k3] += 1;  // counted only when the copy is known complete
      if (kg >= 2 && !bk_wait(b_empty + (kg & 1), (uint32_t)((kg >> 1) - 1) & 1u, abort_flag, polls))
        bad = true;
      // b[c - cw0] = sum_d (w_d x_j) A_j over the taps j of coarse c (zero outside [C0, C1))
      float* b = bbuf(kg & 1);
      const __nv_bfloat16* er = erow(k3);
      int th = ath0, ring = ar0;
      for (int c = sl.cw0 + gt; c < sl.cw1; c += kCfGroup) {
        float v = 0.f;
        if (c >= sl.C0 && c < sl.C1) {
          const int jr = ring * a.ring_len - sl.jw0;  // first fine voxel of the ring, window-relative
          if (th > 0) {
            const int o = jr + 4 * th - 4;  // a multiple of 4: 16-byte x loads, 8-byte A loads
            const float4 x0 = *reinterpret_cast<const float4*>(xs + o), x1 = *reinterpret_cast<const float4*>(xs + o + 4);
            const uint2 a0 = *reinterpret_cast<const uint2*>(er + o), a1 = *reinterpret_cast<const uint2*>(er + o + 4);
            const float xv[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
            const float av[8] = {bf16_lo(a0.x), bf16_hi(a0.x), bf16_lo(a0.y), bf16_hi(a0.y),
                                 bf16_lo(a1.x), bf16_hi(a1.x), bf16_lo(a1.y), bf16_hi(a1.y)};
#pragma unroll
            for (int i = 1; i < 8; ++i) v = fmaf(kW[i] * xv[i], av[i], v);
          } else {
#pragma unroll
            for (int i = 1; i < 8; ++i) {
              const int pj = i - 4 < 0 ? i - 4 + a.ring_len : i - 4;
              v = fmaf(kW[i] * xs[jr + pj], __bfloat162float(er[jr + pj]), v);
            }
          }
        }
        b[c - sl.cw0] = v;
        th += kCfGroup;
        while (th >= nthc) {
          th -= nthc;
          ++ring;
        }
      }
      if (role_sync_or(5, kCfGroup, bad)) {
        aborted = true;
        break;
      }
      if (gt == 0) mbar_arrive(b_full + (kg & 1));
      if (kg >= 1 && !scatter(kg - 1)) {
        aborted = true;
        break;
      }
    }
    if (!aborted && n_mine > 0 && !scatter(n_mine - 1)) aborted = true;
    if (aborted) {
      *abort_flag = 1;
    } else {
      float* out = a.part + (int64_t)cid * a.ldp + sl.J0;
#pragma unroll
      for (int m = 0; m < kCfRuns; ++m) {
        const int rho = gt + m * kCfGroup;
        if (rho < n_runs) *reinterpret_cast<float4*>(out + 4 * rho) = make_float4(acc[m][0], acc[m][1], acc[m][2], acc[m][3]);
      }
    }
  } else {
    // ------------------------------------------------------------ event teams
    const int team = warp / kCfTeamWarps, tw = warp % kCfTeamWarps, lt = tid - team * kCfTeam;
    const int bar_team = 1 + team;  // named barriers 1, 2: one team each
    const int wc = sl.cw1 - sl.cw0;
    float* redt = red + team * kCfTeamWarps * kCfNB;
    float* cst = cs + team * kCfNB;
    float4 qa[kCfQ];
    bool bad = false, aborted = false;
    int bs = 0;   // batch counter over the cluster's groups (both teams count every batch)
    int seq = 0;  // event counter (slot sequence)
    for (int kg = 0; kg < n_mine; ++kg) {
      const int gi = cid + kg * G;
      const int e0 = a.goff[gi], e1 = a.goff[gi + 1];
      if (!bk_wait(b_full + (kg & 1), (uint32_t)(kg >> 1) & 1u, abort_flag, polls)) bad = true;
      const float* b = bbuf(kg & 1);
#pragma unroll
      for (int u = 0; u < kCfQ; ++u) qa[u] = make_float4(0.f, 0.f, 0.f, 0.f);
      for (int eb = e0; eb < e1; eb += kCfNB, ++bs) {
        const int n = min(kCfNB, e1 - eb);
        const int seq_b = seq;
        seq += n;
        if ((bs & 1) != team) continue;  // the other team's batch
        int sk[kCfNB];
#pragma unroll
        for (int k = 0; k < kCfNB; ++k) {
          sk[k] = (seq_b + k) % a.n_slots;
          if (k < n) {
            if (!bk_wait(full + sk[k], (uint32_t)((seq_b + k) / a.n_slots) & 1u, abort_flag, polls))
              bad = true;
            else if (lt == 0)
              slot_waited[sk[k]] += 1;  // counted only when the copy is known complete
          }
        }
        // ---- partial dots over this CTA's window (b is zero outside [C0, C1))
        uint2 rc[kCfNB][kCfQ];
        float4 ac[kCfNB];
#pragma unroll
        for (int k = 0; k < kCfNB; ++k) ac[k] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < kCfQ; ++u) {
          const int c = 4 * lt + u * (4 * kCfTeam);
          if (c < wc) {
            const float4 bv = *reinterpret_cast<const float4*>(b + c);
#pragma unroll
            for (int k = 0; k < kCfNB; ++k)
              if (k < n) {
                rc[k][u] = *reinterpret_cast<const uint2*>(slot(sk[k]) + c);
                ac[k].x = fmaf(bf16_lo(rc[k][u].x), bv.x, ac[k].x);
                ac[k].y = fmaf(bf16_hi(rc[k][u].x), bv.y, ac[k].y);
                ac[k].z = fmaf(bf16_lo(rc[k][u].y), bv.z, ac[k].z);
                ac[k].w = fmaf(bf16_hi(rc[k][u].y), bv.w, ac[k].w);
              }
          }
        }
#pragma unroll
        for (int k = 0; k < kCfNB; ++k)
          if (k < n) {
            const float f = warp_sum((ac[k].x + ac[k].y) + (ac[k].z + ac[k].w));
            if (lane == 0) redt[tw * kCfNB + k] = f;
          }
        if (role_sync_or(bar_team, kCfTeam, bad)) {
          aborted = true;
          break;
        }
        if (lt == 0) {
          // ---- exchange: this CTA's partials to every CTA of the cluster; f = sum in CTA order
          float fr[kCfNB] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
          for (int k = 0; k < kCfNB; ++k)
            if (k < n) {
              float f = 0.f;
              for (int w = 0; w < kCfTeamWarps; ++w) f += redt[w * kCfNB + k];
              fr[k] = f;
            }
          float si[kCfNB] = {1.f, 1.f, 1.f, 1.f};
          if (MODE == 0) {
#pragma unroll
            for (int k = 0; k < kCfNB; ++k)
              if (k < n) si[k] = a.s_ev[eb + k];
          }
          const int x = bs % kCfNX;
          mbar_arrive_expect_tx(xfull + x, (uint32_t)(kCfCluster * kCfNB * sizeof(float)));
          float* dst = xval + (x * kCfCluster + (int)rank) * kCfNB;
          for (uint32_t d = 0; d < (uint32_t)kCfCluster; ++d)
            st_async_v4(map_to_rank(dst, d), fr[0], fr[1], fr[2], fr[3], map_to_rank(xfull + x, d));
          const bool ok = cf_wait_cluster(xfull + x, (uint32_t)(bs / kCfNX) & 1u, abort_flag, polls);
          if (ok) {
#pragma unroll
            for (int k = 0; k < kCfNB; ++k) {
              float f = 0.f;
              for (int r = 0; r < kCfCluster; ++r) f += xval[(x * kCfCluster + r) * kCfNB + k];
              float c = 0.f;
              if (k < n) {
                if (MODE == 0) c = (isfinite(si[k]) && si[k] > 0.f) ? 1.0f / fmaxf(f, 1e-12f * si[k]) : 0.f;
                else c = 1.0f / fmaxf(f, 1e-12f);
              }
              cst[k] = c;
            }
          } else {
            bad = true;
          }
        }
        if (role_sync_or(bar_team, kCfTeam, bad)) {
          aborted = true;
          break;
        }
        // ---- q += c_i t_i over the batch, events in order
#pragma unroll
        for (int k = 0; k < kCfNB; ++k)
          if (k < n) {
            const float ck = cst[k];
            if (ck != 0.f) {
#pragma unroll
              for (int u = 0; u < kCfQ; ++u) {
                const int c = 4 * lt + u * (4 * kCfTeam);
                if (c < wc) {
                  qa[u].x = fmaf(ck, bf16_lo(rc[k][u].x), qa[u].x);
                  qa[u].y = fmaf(ck, bf16_hi(rc[k][u].x), qa[u].y);
                  qa[u].z = fmaf(ck, bf16_lo(rc[k][u].y), qa[u].z);
                  qa[u].w = fmaf(ck, bf16_hi(rc[k][u].y), qa[u].w);
                }
              }
            }
          }
        role_sync(bar_team, kCfTeam);  // the batch's slots, partials and coefficients are free
        if (lt == 0) {
#pragma unroll
          for (int k = 0; k < kCfNB; ++k)
            if (k < n) mbar_arrive(empty + sk[k]);
        }
      }
      if (aborted) break;
      // ---- end of the group: this team's q into its own buffer (the scatter adds the two
      // teams' buffers, team 0 first)
      if (kg >= 2 && !bk_wait(q_empty + (kg & 1), (uint32_t)((kg >> 1) - 1) & 1u, abort_flag, polls)) bad = true;
      if (role_sync_or(bar_team, kCfTeam, bad)) {
        aborted = true;
        break;
      }
      float* q = qbuf(kg & 1, team);
#pragma unroll
      for (int u = 0; u < kCfQ; ++u) {
        const int c = 4 * lt + u * (4 * kCfTeam);
        if (c < wc) *reinterpret_cast<float4*>(q + c) = qa[u];
      }
      role_sync(bar_team, kCfTeam);
      if (lt == 0) {
        mbar_arrive(q_full + (kg & 1));
        mbar_arrive(b_empty + (kg & 1));
      }
    }
    if (aborted) *abort_flag = 1;
  }
  __syncthreads();
  if (*abort_flag && tid == 0) {
    atomicAdd(&g_wait_timeout_count, 1u);
    // bulk copies still in flight write this CTA's shared memory: wait (bounded) for them
    for (int s = 0; s < a.n_slots; ++s)
      if (slot_issued[s] > slot_waited[s])
        mbar_wait_bounded(full + s, (uint32_t)slot_waited[s] & 1u, kBkDrainPolls);
    for (int k = 0; k < 3; ++k)
      if (erow_issued[k] > erow_waited[k])
        mbar_wait_bounded(erow_full + k, (uint32_t)erow_waited[k] & 1u, kBkDrainPolls);
  }
  __syncthreads();
  cluster_sync_all();  // no CTA leaves while a peer may still write its shared memory
}
