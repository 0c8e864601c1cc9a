// Two B-ADMM iterations per HBM pass, for phases whose plans each fit in one
// CTA (included by plan_kernel.cuh).
//
// Iteration t runs in full: its row scale c_w[label] / rowsum(Z') needs only
// the CTA's own columns and c_w as it stands after iteration t-1, which the
// cluster reduction has produced before the pass.  Iteration t+1 then runs
// step 1 and the first half of step 2 on the Z and Y of iteration t, still in
// registers, and leaves deferred: Z' and U = Y + X are stored with the raw row
// sums of Z' (its step-4 row sums too).  Once the cluster reduction of
// iteration t has produced c_w, pair_scale_kernel forms the row scale
// c_w / rowsum(Z') of every plan, and the next pass (or pair_finalize_kernel)
// applies it on load: Z = Z' * scale, Y = U - Z.  Z and Y cross HBM once per two
// iterations; the arithmetic per entry is that of two single passes, except
// that the deferred Y is rounded twice (U, then U - Z).
//
// The host pairs iterations (t, t+1) only where this is exact: t is no
// support-update iteration (its update would change the costs of t+1), t+1 is
// no residual-check iteration (its check needs the final Z of t+1), and no
// time budget is set (the reference may stop after any single iteration).
//
// flags: PF_IN_DEF   the input is deferred: every plan's row scale in a.rowsc [plan][MP]
//                     (packed order: the plans of a unit are contiguous)
//        PF_STAGE_SC each unit's row scales arrive with its tiles (bulk copy into
//                     shared memory, the same transaction); else read per thread
//        PF_UPDATE   iteration t+1 is a Euclidean support update: its X moments
//        PF_WRITE_X  iteration t+1's X is stored (word-embedding support update)
// CHECK: iteration t is a residual-check iteration.
#pragma once

namespace d2g {

// seg_sum over the TPC lanes of this thread's aligned segment, with only those
// lanes taking part (callable where other segments of the warp diverge)
template <int TPC>
__device__ __forceinline__ float seg_sum_lanes(float v) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned mask = TPC == 32 ? 0xffffffffu : (((1u << TPC) - 1u) << (lane & ~(unsigned)(TPC - 1)));
#pragma unroll
  for (int o = TPC / 2; o >= 1; o >>= 1) v += __shfl_xor_sync(mask, v, o);
  return v;
}

template <int MP, int MODE, bool CHECK, bool FULL>
__global__ void __launch_bounds__(GeoT<MP>::NT, 2) plan_pair_kernel(const PlanArgs a, int nitems) {
  using T = Tile<MP, MODE>;
  constexpr int RPT = T::RPT, TPC = T::TPC, G = T::G, S = T::S;
  constexpr int TILE = tma_tile_floats<MP>();
  constexpr int JC = G * S;
  constexpr int CW = T::EUC ? T::DS : 1;
  constexpr bool SCC = plan_stages_costs(MP, MODE);
  constexpr int CPR = MP / 4;
  constexpr int NT = GeoT<MP>::NT;
  constexpr int PPT = SCC ? TILE / 4 / NT : 1;
  const bool SC = SCC && a.stage_costs;
  extern __shared__ __align__(128) float smem[];
  float *stZ = smem;                             // [2][TILE]
  float *stY = smem + 2 * TILE;                  // [2][TILE]
  int4 *stR = (int4 *)(smem + 4 * TILE);         // [2][G] group records
  float *stW = (float *)(stR + 2 * G);           // [2][JC] weights
  float *stC = stW + 2 * JC;                     // [2][JC*CW] supports / table rows
  float *stK = stC + 2 * JC * CW;                // [2][TILE] staged table costs (SC)
  float *sm_rs = stK + (SCC ? 2 * TILE : 0);     // [G][MP] row partials of iteration t
  float *sm_rs2 = sm_rs + G * MP;                // [G][MP] row partials of iteration t+1
  float *sm_mom = sm_rs2 + G * MP;               // [dim+1][G][MP] X moments of iteration t+1
  float *stS = sm_mom + (a.dim + 1) * G * MP;    // [2][G][MP] row scales of the unit's plans
  __shared__ __align__(8) unsigned long long mbar[2];
  __shared__ int sh_fail;
  __shared__ int sh_g0[2], sh_ng[2];
  __shared__ int2 sh_pp[2];

  if (a.iter >= a.ctl->stop_iter) return;
  const int tid = threadIdx.x;
  const int u0 = blockIdx.x, ustep = gridDim.x, nunits = nitems;
  if (a.iter == 0 && blockIdx.x == 0 && tid == 0) a.ctl->t_start_ns = global_ns();
  const unsigned long long wlim = wait_limit(a.ctl);
  const int fault_u = withheld_unit(a.ctl, a.iter);
  const bool indef = a.flags & PF_IN_DEF;
  const bool stage_sc = indef && (a.flags & PF_STAGE_SC);
  // The plans {first, count} of unit u (thread 0).  Thread 0 loads the
  // bounds of a unit one unit before it issues that unit's copy, and checks
  // them only then: any use of a loaded value right after the load would stall
  // warp 0, and with it every warp at the unit's next barrier.
  auto unit_plans = [&](int u) { return indef ? a.item_pp[u] : make_int2(0, 0); };
  auto checked = [&](int2 pp) {
    if (pp.x < 0 || pp.y < 0 || pp.y > G || pp.x > a.nplans_chk - pp.y) {
      ctl_fail(a.ctl, 9);
      pp = make_int2(0, 0);
    }
    return pp;
  };
  auto issue = [&](int unit, int g0, int ng, int2 pp, int stg) {
    const size_t off = (size_t)g0 * S * MP;
    const unsigned bytes = (unsigned)ng * S * MP * 4u;
    const unsigned rb = (unsigned)ng * 16u, wb = (unsigned)ng * S * 4u, cb = wb * CW;
    const unsigned sb = stage_sc && ng > 0 ? (unsigned)pp.y * MP * 4u : 0u;
    mbar_expect_tx(&mbar[stg], 2u * bytes + rb + wb + cb + sb);
    if (ng <= 0) return;
    if (unit == fault_u) return;  // test hook: the stage's transaction never completes
    if (sb) bulk_load(stS + stg * G * MP, a.rowsc + (size_t)pp.x * MP, sb, &mbar[stg]);
    bulk_load(stZ + stg * TILE, a.Z + off, bytes, &mbar[stg]);
    bulk_load(stY + stg * TILE, a.Y + off, bytes, &mbar[stg]);
    bulk_load(stR + stg * G, a.grp_rec + g0, rb, &mbar[stg]);
    bulk_load(stW + stg * JC, a.col_w + (size_t)g0 * S, wb, &mbar[stg]);
    if constexpr (T::EUC)
      bulk_load(stC + stg * JC * CW, a.col_supp + (size_t)g0 * S * CW, cb, &mbar[stg]);
    else
      bulk_load(stC + stg * JC * CW, a.col_sym + (size_t)g0 * S, cb, &mbar[stg]);
  };
  int crow_p[PPT];
  auto load_rows_idx = [&](int g0, int ng) {
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
      const int c = (tid + NT * j) / CPR;
      crow_p[j] = c < ng * S ? __ldg(a.col_crow + (size_t)g0 * S + c) : -1;
    }
  };
  auto issue_rows = [&](int stg) {
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
      const int i = tid + NT * j, c = i / CPR, part = i - c * CPR;
      // (the row index is checked here, where the loaded value is consumed
      // anyway: a row outside the table is reported, not read)
      if (crow_p[j] >= a.ctab_rows) ctl_fail(a.ctl, 9);
      else if (crow_p[j] >= 0)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(
                         smem_u32(stK + stg * TILE + c * MP + part * 4)),
                     "l"(a.ctab + (size_t)crow_p[j] * MP + part * 4)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  int nx_g0 = 0, nx_ng = 0;
  int2 nx_pp = make_int2(0, 0);
  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    sh_fail = 0;
    mbar_fence_init();
    if (u0 < nunits) {
      const int g0 = a.item_g0[u0], ng = a.item_ng[u0];
      const int2 pp = checked(unit_plans(u0));
      sh_g0[0] = g0;
      sh_ng[0] = ng;
      sh_pp[0] = pp;
      issue(u0, g0, ng, pp, 0);
      if (u0 + ustep < nunits) {
        nx_g0 = a.item_g0[u0 + ustep];
        nx_ng = a.item_ng[u0 + ustep];
        nx_pp = unit_plans(u0 + ustep);
      }
    }
  }
  if (SC && u0 < nunits) {
    __syncthreads();
    load_rows_idx(sh_g0[0], sh_ng[0]);
    issue_rows(0);
  }
  __syncthreads();

  const int m = a.m;
  const float inv_rho = a.ctl->inv_rho;
  const float ir2 = a.ctl->inv_rho_l2;
  const bool update = T::EUC && (a.flags & PF_UPDATE);
  const bool write_x = a.flags & PF_WRITE_X;
  double s_obj = 0.0, s_pr = 0.0, s_dr = 0.0;
  int it = 0;
  for (int u = u0; u < nunits; u += ustep, ++it) {
    const int stg = it & 1;
    if (!mbar_wait(&mbar[stg], (it >> 1) & 1, wlim)) sh_fail = 1;
    if (SC) asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    if (sh_fail) break;
    const int cur_g0 = sh_g0[stg], cur_ng = sh_ng[stg];
    const int2 cur_pp = sh_pp[stg];
    if (tid == 0 && u + ustep < nunits) {
      nx_pp = checked(nx_pp);
      issue(u + ustep, nx_g0, nx_ng, nx_pp, stg ^ 1);
      sh_g0[stg ^ 1] = nx_g0;
      sh_ng[stg ^ 1] = nx_ng;
      sh_pp[stg ^ 1] = nx_pp;
      if (u + 2 * ustep < nunits) {
        nx_g0 = a.item_g0[u + 2 * ustep];
        nx_ng = a.item_ng[u + 2 * ustep];
        nx_pp = unit_plans(u + 2 * ustep);
      }
    }
    const bool has_next = u + ustep < nunits;

    T t;
    t.init_rec(stR[stg * G + (threadIdx.x / TPC)], cur_g0, cur_ng);
    // self-check of the staged group record: a plan inside this unit, a slot
    // and label inside the phase, the plan among the unit's row scales (a bad
    // record is reported and its group idles)
    if (t.active && (t.p < 0 || t.p >= a.nplans_chk || t.lab < 0 || t.lab >= a.nlab_chk ||
                     t.pl_g0 < cur_g0 || t.pl_g0 + t.pl_ng > cur_g0 + cur_ng || t.pl_ng < 1 ||
                     (indef && t.lp >= cur_pp.y))) {
      ctl_fail(a.ctl, 9);
      t.active = false;
      t.nvalid = 0;
      t.p = 0;
      t.lab = 0;
      t.pl_g0 = cur_g0;
      t.pl_ng = 0;
    }
    t.load_costs_staged(a, stC + stg * JC * CW, (const int *)(stC + stg * JC * CW));
    const float *zs = stZ + stg * TILE, *ys = stY + stg * TILE;
    const int lcol0 = t.g * S;
    float w[S];
#pragma unroll
    for (int s = 0; s < S; ++s) w[s] = s < t.nvalid ? stW[stg * JC + lcol0 + s] : 0.f;
    // deferred input: this plan's row scale (plan cur_pp.x + t.lp in packed order)
    float scin[RPT];
#pragma unroll
    for (int q4 = 0; q4 < RPT / 4; ++q4) {
      float4 v = make_float4(1.f, 1.f, 1.f, 1.f);
      if (stage_sc && t.active)
        v = *((const float4 *)(stS + (stg * G + t.lp) * MP + t.k0) + q4);
      else if (indef && t.active)
        v = __ldg((const float4 *)(a.rowsc + (size_t)(cur_pp.x + t.lp) * MP + t.k0) + q4);
      scin[4 * q4] = v.x;
      scin[4 * q4 + 1] = v.y;
      scin[4 * q4 + 2] = v.z;
      scin[4 * q4 + 3] = v.w;
    }
    auto ld_zy = [&](int s, float (&z)[RPT], float (&y)[RPT]) {
#pragma unroll
      for (int q4 = 0; q4 < RPT / 4; ++q4) {
        const float4 zz = *((const float4 *)(zs + (lcol0 + s) * MP + t.k0) + q4);
        const float4 yy = *((const float4 *)(ys + (lcol0 + s) * MP + t.k0) + q4);
        z[4 * q4] = zz.x; z[4 * q4 + 1] = zz.y; z[4 * q4 + 2] = zz.z; z[4 * q4 + 3] = zz.w;
        y[4 * q4] = yy.x; y[4 * q4 + 1] = yy.y; y[4 * q4 + 2] = yy.z; y[4 * q4 + 3] = yy.w;
      }
      if (indef) {
#pragma unroll
        for (int h = 0; h < RPT / 2; ++h) {
          const float2 zz = __fmul2_rn(pr2(z, h), pr2(scin, h));
          st2(z, h, zz);
          st2(y, h, __ffma2_rn(bc2(-kLog2e), zz, pr2(y, h)));
        }
      }
    };
    auto costs = [&](int s, float (&c)[RPT]) {
      if (SC) {
#pragma unroll
        for (int q4 = 0; q4 < RPT / 4; ++q4) {
          const float4 v = *((const float4 *)(stK + stg * TILE + (lcol0 + s) * MP + t.k0) + q4);
          c[4 * q4] = v.x; c[4 * q4 + 1] = v.y; c[4 * q4 + 2] = v.z; c[4 * q4 + 3] = v.w;
        }
      } else {
        t.costs(s, c);
      }
    };
    // steps 1 and 2 up to Z' of one column: x (X), zp (Z'); returns nothing, fills arrays
    auto half = [&](int s, const float (&c)[RPT], const float (&z)[RPT], const float (&y)[RPT],
                    float (&x)[RPT], float (&zp)[RPT]) {
      const bool colok = s < t.nvalid;
      float2 vs = bc2(0.f);
#pragma unroll
      for (int h = 0; h < RPT / 2; ++h) {
        float2 v = __ffma2_rn(pr2(z, h), nex2f2(__ffma2_rn(pr2(c, h), bc2(ir2), pr2(y, h))), bc2(kRoundoff));
        if constexpr (!FULL) {
          if (!(colok && t.k0 + 2 * h < m)) v.x = 0.f;
          if (!(colok && t.k0 + 2 * h + 1 < m)) v.y = 0.f;
        }
        st2(x, h, v);
        vs = h == 0 ? v : __fadd2_rn(vs, v);
      }
      const float csum = seg_sum<TPC>(vs.x + vs.y);
      const float f = (FULL || colok) ? __fdividef(w[s], csum) : 0.f;
      const float eps2 = colok ? kRoundoff : 0.f;
#pragma unroll
      for (int h = 0; h < RPT / 2; ++h) {
        const float2 xv = __fmul2_rn(pr2(x, h), bc2(f));
        float2 zz = __ffma2_rn(xv, ex2f2(pr2(y, h)), bc2(eps2));
        if constexpr (!FULL) {
          if (!(t.k0 + 2 * h < m)) zz.x = 0.f;
          if (!(t.k0 + 2 * h + 1 < m)) zz.y = 0.f;
        }
        st2(x, h, xv);
        st2(zp, h, zz);
      }
    };
    // the plan totals of the row partials in buf: the first group of each plan
    // sums them once and publishes the total in place of its own partial
    const int lo = t.active ? max(t.pl_g0 - t.cta_g0, 0) : 0;
    const int hi = t.active ? min(t.pl_g0 + t.pl_ng - t.cta_g0, t.cta_ng) : 0;
    const bool writer = t.active && t.g == lo;

    // ---------------- iteration t: steps 1-3 in full
    float x[S][RPT], zp[S][RPT];
#pragma unroll
    for (int s = 0; s < S; ++s) {
      float c[RPT], z[RPT], y[RPT];
      costs(s, c);
      ld_zy(s, z, y);
      half(s, c, z, y, x[s], zp[s]);
    }
    {
      float rp[RPT];
#pragma unroll
      for (int h = 0; h < RPT / 2; ++h) {
        float2 u = pr2(zp[0], h);
#pragma unroll
        for (int s = 1; s < S; ++s) u = __fadd2_rn(u, pr2(zp[s], h));
        st2(rp, h, u);
      }
      st_rows_sm(sm_rs + t.g * MP + t.k0, rp);
    }
    __syncthreads();
    if (SC && has_next) load_rows_idx(sh_g0[stg ^ 1], sh_ng[stg ^ 1]);
    // c_w of the plan's cluster for iteration t's row scale, read before the
    // totals barrier so that its latency overlaps the wait
    float cwv[RPT];
#pragma unroll
    for (int q4 = 0; q4 < RPT / 4; ++q4) {
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (t.active) v = __ldg((const float4 *)(a.cw32 + (size_t)t.lab * MP + t.k0) + q4);
      cwv[4 * q4] = v.x;
      cwv[4 * q4 + 1] = v.y;
      cwv[4 * q4 + 2] = v.z;
      cwv[4 * q4 + 3] = v.w;
    }
    float tot[RPT];
    if (writer) {
#pragma unroll
      for (int q = 0; q < RPT; ++q) tot[q] = 0.f;
      for (int j = lo; j < hi; ++j) {
#pragma unroll
        for (int q4 = 0; q4 < RPT / 4; ++q4) {
          const float4 u4 = *((const float4 *)(sm_rs + j * MP + t.k0) + q4);
          tot[4 * q4] += u4.x;
          tot[4 * q4 + 1] += u4.y;
          tot[4 * q4 + 2] += u4.z;
          tot[4 * q4 + 3] += u4.w;
        }
      }
      st_rows_sm(sm_rs + lo * MP + t.k0, tot);
    }
    __syncthreads();
#pragma unroll
    for (int q4 = 0; q4 < RPT / 4; ++q4) {
      const float4 u4 = *((const float4 *)(sm_rs + lo * MP + t.k0) + q4);
      tot[4 * q4] = u4.x;
      tot[4 * q4 + 1] = u4.y;
      tot[4 * q4 + 2] = u4.z;
      tot[4 * q4 + 3] = u4.w;
    }
    {
      float rsum = 0.f;  // step 4's per-instance normalisation of Zr (:180)
#pragma unroll
      for (int q = 0; q < RPT; ++q) rsum += (FULL || t.k0 + q < m) ? tot[q] : 0.f;
      rsum = seg_sum<TPC>(rsum);
      if (writer) {
        float zr[RPT];
        const float inv = 1.f / rsum;
#pragma unroll
        for (int q = 0; q < RPT; ++q) zr[q] = tot[q] * inv;
        st_rows(a.rowsum_out + (size_t)t.p * MP + t.k0, zr);
      }
    }
    float sc[RPT];
#pragma unroll
    for (int q = 0; q < RPT; ++q) {
      const bool ok = t.active && (FULL || t.k0 + q < m);
      sc[q] = ok ? __fdividef(cwv[q], tot[q]) : 0.f;
    }
    // second half of step 2 and step 3: Z and Y of iteration t stay in registers
    float zt[S][RPT], yt[S][RPT];
    float i_obj = 0.f, i_pr = 0.f, i_dr = 0.f;
#pragma unroll
    for (int s = 0; s < S; ++s) {
      float z0[RPT], y[RPT];
      ld_zy(s, z0, y);
      const bool colok = s < t.nvalid;
#pragma unroll
      for (int h = 0; h < RPT / 2; ++h) {
        const float2 zn = __fmul2_rn(pr2(zp[s], h), pr2(sc, h));
        // (x - zn as fma(zn, -1, x): the same single rounding)
        const float2 yn = __ffma2_rn(bc2(kLog2e), __ffma2_rn(zn, bc2(-1.f), pr2(x[s], h)), pr2(y, h));
        st2(zt[s], h, colok ? zn : bc2(0.f));
        st2(yt[s], h, colok ? yn : bc2(0.f));
      }
      if constexpr (CHECK) {
        if (colok) {
          float c[RPT];
          costs(s, c);
#pragma unroll
          for (int q = 0; q < RPT; ++q) {
            i_obj = fmaf(c[q] * inv_rho, x[s][q], i_obj);
            i_pr += fabsf(x[s][q] - zt[s][q]);
            i_dr += fabsf(zt[s][q] - z0[q]);
          }
        }
      }
    }
    if constexpr (CHECK) {
      s_obj += i_obj;
      s_pr += i_pr;
      s_dr += i_dr;
    }

    // ---------------- iteration t+1: steps 1 and 2 up to Z', deferred output
#pragma unroll
    for (int s = 0; s < S; ++s) {
      float c[RPT];
      costs(s, c);
      half(s, c, zt[s], yt[s], x[s], zp[s]);
      if (s < t.nvalid) {
        float un[RPT];
#pragma unroll
        for (int h = 0; h < RPT / 2; ++h)  // U = Y + X
          st2(un, h, __ffma2_rn(bc2(kLog2e), pr2(x[s], h), pr2(yt[s], h)));
        const size_t off = (t.colbase + s) * MP + t.k0;
        st_rows(a.Z + off, zp[s]);
        st_rows(a.Y + off, un);
        if (write_x) st_rows(a.X_out + off, x[s]);
      }
    }
    {
      float rp[RPT];
#pragma unroll
      for (int h = 0; h < RPT / 2; ++h) {
        float2 u = pr2(zp[0], h);
#pragma unroll
        for (int s = 1; s < S; ++s) u = __fadd2_rn(u, pr2(zp[s], h));
        st2(rp, h, u);
      }
      st_rows_sm(sm_rs2 + t.g * MP + t.k0, rp);
    }
    if constexpr (T::EUC) {
      if (update) {  // X moments of iteration t+1 (step 5)
        for (int d = 0; d <= a.dim; ++d) {
          float mv[RPT];
#pragma unroll
          for (int q = 0; q < RPT; ++q) {
            float acc = 0.f;
#pragma unroll
            for (int s = 0; s < S; ++s) {
              float sv = 1.f;
              if (d < a.dim) {
#pragma unroll
                for (int tt = 0; tt < T::DS; ++tt)
                  if (tt == d) sv = t.sp[s][tt];
              }
              acc = fmaf(x[s][q], sv, acc);
            }
            mv[q] = acc;
          }
          st_rows_sm(sm_mom + (d * G + t.g) * MP + t.k0, mv);
        }
      }
    }
    __syncthreads();
    if (writer) {
      float tot2[RPT];
#pragma unroll
      for (int q = 0; q < RPT; ++q) tot2[q] = 0.f;
      for (int j = lo; j < hi; ++j) {
#pragma unroll
        for (int q4 = 0; q4 < RPT / 4; ++q4) {
          const float4 u4 = *((const float4 *)(sm_rs2 + j * MP + t.k0) + q4);
          tot2[4 * q4] += u4.x;
          tot2[4 * q4 + 1] += u4.y;
          tot2[4 * q4 + 2] += u4.z;
          tot2[4 * q4 + 3] += u4.w;
        }
      }
      st_rows(a.rawsum_out + (size_t)t.p * MP + t.k0, tot2);
      float rsum = 0.f;
#pragma unroll
      for (int q = 0; q < RPT; ++q) rsum += (FULL || t.k0 + q < m) ? tot2[q] : 0.f;
      // the writer threads of one plan are the TPC threads of its first group,
      // one aligned segment of the warp: the sum runs among those lanes only
      rsum = seg_sum_lanes<TPC>(rsum);
      float zr[RPT];
      const float inv = 1.f / rsum;
#pragma unroll
      for (int q = 0; q < RPT; ++q) zr[q] = tot2[q] * inv;
      st_rows(a.rowsum2_out + (size_t)t.p * MP + t.k0, zr);
      if (T::EUC && update) {
        float *xo = a.xmom_out + (size_t)t.p * (a.dim + 1) * MP;
        for (int d = 0; d <= a.dim; ++d) {
          float mv[RPT];
#pragma unroll
          for (int q = 0; q < RPT; ++q) mv[q] = 0.f;
          for (int j = lo; j < hi; ++j)
#pragma unroll
            for (int q = 0; q < RPT; ++q) mv[q] += sm_mom[(d * G + j) * MP + t.k0 + q];
          st_rows(xo + d * MP + t.k0, mv);
        }
      }
    }
    if (SC && has_next) issue_rows(stg ^ 1);
    // No barrier here: the next unit's opening barrier orders every reuse of
    // the stage, the row partials and the staged rows.
  }
  if (SC) asm volatile("cp.async.wait_all;" ::: "memory");
  if (sh_fail) {
    if (tid == 0) {
      ctl_fail(a.ctl, 7);
      // the one copy that can be in flight is the failed unit's (it): stage
      // it & 1, phase parity (it >> 1) & 1 (the next stage is issued only
      // after a successful wait); wait for it once more, bounded
      mbar_wait(&mbar[it & 1], (it >> 1) & 1, wlim);
    }
    return;
  }
  if constexpr (CHECK) {
    __shared__ double res[3];
    block_sum3<NT>(s_obj, s_pr, s_dr, res);
    if (tid == 0 && u0 < nitems) {
      double *pp = a.resid_part + (size_t)(a.resid_off + u0) * 4;
      pp[0] = res[0];
      pp[1] = res[1];
      pp[2] = res[2];
      for (int item = u0 + ustep; item < nitems; item += ustep) {
        double *qq = a.resid_part + (size_t)(a.resid_off + item) * 4;
        qq[0] = qq[1] = qq[2] = 0.0;
      }
    }
  }
}

// shared memory of plan_pair_kernel beyond its static part (without the
// staged row scales of pair_scale_bytes)
template <int MP>
size_t pair_smem_bytes(int mode, int dim) {
  using Gm = GeoT<MP>;
  const int cw = mode == COST_TABLE ? 1 : (mode == COST_EUCLID8 ? 8 : 4);
  return (size_t)4 * tma_tile_floats<MP>() * 4 + 2 * (size_t)Gm::G * 16 + 2 * (size_t)Gm::JC * 4 * (1 + cw) +
         (plan_stages_costs(MP, mode) ? (size_t)2 * tma_tile_floats<MP>() * 4 : 0) +
         (size_t)2 * Gm::G * MP * 4 + (size_t)(dim + 1) * Gm::G * MP * 4;
}

// two stages of row scales, one row per plan of a unit (at most G plans)
template <int MP>
constexpr size_t pair_scale_bytes() {
  return (size_t)2 * GeoT<MP>::G * MP * 4;
}

// The row scales of deferred input are staged in shared memory when that
// keeps the CTAs per SM of the unstaged kernel; otherwise each thread reads
// its plan's scale from global memory.
template <int MP, int MODE, bool CHECK, bool FULL>
cudaError_t launch_pair_t(const PlanArgs &a, int nitems, cudaStream_t st) {
  static std::mutex mu;  // the cached launch shapes are shared by phases on other host threads
  std::lock_guard<std::mutex> lk(mu);
  struct Shape {
    int grid = 0, nsm = 0;
    bool stage = false;
    size_t configured = 0;
  };
  static Shape shapes[kMaxDevices];
  int dev = 0;
  if (cudaError_t e = launch_device(&dev); e != cudaSuccess) return e;
  Shape &sh = shapes[dev];
  const size_t sm0 = pair_smem_bytes<MP>(MODE, a.dim), sm1 = sm0 + pair_scale_bytes<MP>();
  auto kern = plan_pair_kernel<MP, MODE, CHECK, FULL>;
  if (sh.configured < sm1) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1);
    if (e != cudaSuccess) {  // beyond the opt-in limit: the kernel without staged scales
      (void)cudaGetLastError();
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm0);
      if (e != cudaSuccess) return e;
      sh.configured = sm0;
      sh.stage = false;
    } else {
      sh.configured = sm1;
    }
    sh.grid = 0;
  }
  if (sh.grid == 0) {
    int per0 = 0, per1 = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sh.nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per0, kern, GeoT<MP>::NT, sm0);
    if (e == cudaSuccess && sh.configured >= sm1)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, kern, GeoT<MP>::NT, sm1);
    if (e != cudaSuccess) return e;
    sh.stage = sh.configured >= sm1 && per1 >= per0;
    const int per = sh.stage ? per1 : per0;
    sh.grid = (per > 0 ? per : 1) * sh.nsm;
  }
  if (nitems <= 0) return cudaSuccess;
  int cap = sh.grid;
  if (a.ctas_per_sm > 0) cap = std::min(cap, a.ctas_per_sm * sh.nsm);
  const int g = nitems < cap ? nitems : cap;
  PlanArgs b = a;
  if (sh.stage && a.stage_scales && (a.flags & PF_IN_DEF)) b.flags |= PF_STAGE_SC;
  const size_t sm = (b.flags & PF_STAGE_SC) ? sm1 : sm0;
  cudaLaunchAttribute attr[1];
  cudaLaunchConfig_t cfg = plan_cfg(g, GeoT<MP>::NT, sm, st, attr, 1);
  return cudaLaunchKernelEx(&cfg, kern, b, nitems);
}

template <int MP, int MODE, bool CHECK>
cudaError_t launch_pair_c(const PlanArgs &a, int nitems, cudaStream_t st) {
  if (a.m == MP) return launch_pair_t<MP, MODE, CHECK, true>(a, nitems, st);
  return launch_pair_t<MP, MODE, CHECK, false>(a, nitems, st);
}

// the pair kernel exists for MP <= 128: 256-row plans are always wider than a CTA
template <int MP>
cudaError_t launch_pair_mp(int mode, bool check, const PlanArgs &a, int nitems, cudaStream_t st) {
  if constexpr (MP >= 256) {
    return cudaErrorInvalidValue;
  } else {
    if (mode == COST_EUCLID3)
      return check ? launch_pair_c<MP, COST_EUCLID3, true>(a, nitems, st)
                   : launch_pair_c<MP, COST_EUCLID3, false>(a, nitems, st);
    if (mode == COST_EUCLID4)
      return check ? launch_pair_c<MP, COST_EUCLID4, true>(a, nitems, st)
                   : launch_pair_c<MP, COST_EUCLID4, false>(a, nitems, st);
    if (mode == COST_EUCLID8)
      return check ? launch_pair_c<MP, COST_EUCLID8, true>(a, nitems, st)
                   : launch_pair_c<MP, COST_EUCLID8, false>(a, nitems, st);
    return check ? launch_pair_c<MP, COST_TABLE, true>(a, nitems, st)
                 : launch_pair_c<MP, COST_TABLE, false>(a, nitems, st);
  }
}

}  // namespace d2g
