// Runtime dispatch from the padded support size MP to the per-MP kernel
// instantiations (plan_mp*.cu).
#include "d2g_internal.cuh"

namespace d2g {

template <int MP>
cudaError_t launch_plan_mp(int, bool, const PlanArgs &, int, size_t, cudaStream_t);
template <int MP>
cudaError_t launch_rho_mp(int, const PlanArgs &, int, double *, cudaStream_t);
template <int MP>
cudaError_t launch_convert_mp(int, const PlanArgs &, int, double *, const long long *,
                              const char *, const double *, int, cudaStream_t);
template <int MP>
cudaError_t launch_pack_columns_mp(const PlanArgs &, int, const long long *, const double *,
                                   const double *, const int *, float *, float *, int *, int,
                                   int, int, cudaStream_t);
template <int MP>
cudaError_t launch_obj_mp(int, const PlanArgs &, int, cudaStream_t);
template <int MP>
cudaError_t launch_pair_mp(int, bool, const PlanArgs &, int, cudaStream_t);

#define D2G_MP_SWITCH(MPV, CALL) \
  switch (MPV) {                 \
    case 4: return CALL(4);      \
    case 8: return CALL(8);      \
    case 16: return CALL(16);    \
    case 32: return CALL(32);    \
    case 64: return CALL(64);    \
    case 128: return CALL(128);  \
    case 256: return CALL(256);  \
    default: return cudaErrorInvalidValue; \
  }

Geo geo_for(int MP) {
  Geo g;
  g.MP = MP;
  g.RPT = MP >= 256 ? 8 : 4;
  g.TPC = MP / g.RPT;
  g.S = plan_cols_per_thread(MP);
  g.NT = plan_threads(MP);
  g.G = g.NT / g.TPC;
  g.JC = g.G * g.S;
  return g;
}

size_t plan_smem_bytes(int MP, int dim, int cs) {
  (void)cs;
  const Geo g = geo_for(MP);
  const size_t rows = (size_t)g.G * MP + MP;             // row partials + cluster exchange
  const size_t mom = (size_t)(dim + 1) * ((size_t)g.G * MP + MP);  // moments + exchange
  return (rows + mom) * sizeof(float);
}

cudaError_t launch_plan(int MP, int mode, bool check, const PlanArgs &a, int nitems, size_t smem,
                        cudaStream_t st) {
#define C_(X) launch_plan_mp<X>(mode, check, a, nitems, smem, st)
  D2G_MP_SWITCH(MP, C_)
#undef C_
}

cudaError_t launch_rho_partial(int MP, int mode, const PlanArgs &a, int nitems, double *part,
                               cudaStream_t st) {
#define C_(X) launch_rho_mp<X>(mode, a, nitems, part, st)
  D2G_MP_SWITCH(MP, C_)
#undef C_
}

cudaError_t launch_pack_convert(int MP, int dir, const PlanArgs &a, int nitems, double *ref,
                                const long long *plan_refcol, const char *plan_reinit,
                                const double *cw64, int str, cudaStream_t st) {
#define C_(X) launch_convert_mp<X>(dir, a, nitems, ref, plan_refcol, plan_reinit, cw64, str, st)
  D2G_MP_SWITCH(MP, C_)
#undef C_
}

cudaError_t launch_pack_columns(int MP, const PlanArgs &a, int nitems, const long long *plan_cum,
                                const double *w_ref, const double *supp_ref, const int *sym_ref,
                                float *col_w, float *col_supp, int *col_sym, int dim, int DS,
                                int dense_hist, cudaStream_t st) {
#define C_(X)                                                                                   \
  launch_pack_columns_mp<X>(a, nitems, plan_cum, w_ref, supp_ref, sym_ref, col_w, col_supp,    \
                            col_sym, dim, DS, dense_hist, st)
  D2G_MP_SWITCH(MP, C_)
#undef C_
}

cudaError_t launch_plan_pair(int MP, int mode, bool check, const PlanArgs &a, int nitems, cudaStream_t st) {
#define C_(X) launch_pair_mp<X>(mode, check, a, nitems, st)
  D2G_MP_SWITCH(MP, C_)
#undef C_
}

cudaError_t launch_obj(int MP, int mode, const PlanArgs &a, int nitems, cudaStream_t st) {
#define C_(X) launch_obj_mp<X>(mode, a, nitems, st)
  D2G_MP_SWITCH(MP, C_)
#undef C_
}

}  // namespace d2g
