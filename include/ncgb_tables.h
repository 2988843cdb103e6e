/*
 * ncgb_tables.h -- flat, pointer-based view of one material's scattering
 * tables, as laid out in device memory (HBM) by the host table builder.
 *
 * The same structs describe the tables in host memory, so the CPU oracle and
 * the CUDA kernels read one layout.  Plain C, no CUDA or torch types.
 *
 * A material is NCrystal's ProcComposition for one cfg-string
 * (NCProcImpl.hh:310-373): up to NCGB_MAX_COMP components, each with a scale,
 * an energy domain [elow,ehigh] and a type-specific table set:
 *
 *   PowderBragg  two_dE[n], fdm_commul[n]            (NCPowderBragg.hh:29-95)
 *   ElIncScatter (msd, sigma*scale) per element       (NCElIncXS.hh:127)
 *   SABScatter   energy grid + xs, S/logS/cumulative alpha integrals on the
 *                (beta, alpha) grid, one Alg.1 sampler per energy-grid point
 *                (NCSABSampler.hh:91-98, NCSABSamplerModels.hh:31-79)
 *   FreeGas      kT, target mass, sigma_free          (NCFreeGas.cc:25-42)
 */
#ifndef NCGB_TABLES_H
#define NCGB_TABLES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NCGB_MAX_COMP 8
#define NCGB_MAX_ELINC 16

enum ncgb_comp_type {
  NCGB_COMP_NONE = 0,
  NCGB_COMP_ELINC = 1,
  NCGB_COMP_BRAGG = 2,
  NCGB_COMP_SAB = 3,
  NCGB_COMP_FREEGAS = 4
};

/* One beta row's alpha sampler at one energy-grid point
 * (SABSamplerAtE_Alg1::AlphaSampleInfo, NCSABSamplerModels.hh:46-56), plus
 * three reciprocals the GPU uses instead of divisions. */
typedef struct {
  double front_alpha, front_sval, front_logsval;
  double back_alpha, back_sval, back_logsval;
  double prob_front;   /* 1.0: narrow range, 2.0: zero xs (sample linearly) */
  double prob_notback; /* prob_front + prob_middle */
  uint32_t front_idx, back_idx;
  double inv_front;    /* 1/prob_front */
  double inv_middle;   /* 1/(prob_notback-prob_front) */
  double inv_back;     /* 1/(1-prob_notback) */
} ncgb_alpha_info;

/* FP32 copy of ncgb_alpha_info for the mixed-precision mode. */
typedef struct {
  float front_alpha, front_sval, front_logsval;
  float back_alpha, back_sval, back_logsval;
  float prob_front, prob_notback;
  float inv_front, inv_middle, inv_back;
  uint32_t front_idx, back_idx;
  float pad[3];
} ncgb_alpha_info_f;

/* One bin [x0,x1] of a beta sampler's piecewise-linear density, with the
 * constants of PointwiseDist::percentileWithIndex's in-bin inversion
 * (NCPointwiseDist.cc:84-109) precomputed: a = y0, d = y1-y0, dx = x1-x0,
 * k_e = d/(dx*a*a) (a != 0) or 2*dx/d (a == 0, d > 0) or -1, k_z = dx*a/d,
 * inv_a = 1/a. */
typedef struct {
  double x0, x1, cdf0, a;
  double k_e, k_z, inv_a, pad;
} ncgb_beta_bin;

/* Learned beta proposal of one sampler (egrid point): a partition of the
 * sampler's regular beta range into NCGB_LP_K intervals placed from a trained
 * network's quantiles, a piecewise-constant envelope (the maximum of the
 * sampler's piecewise-linear beta density on each interval), an alias table
 * over the interval masses, and per interval the density's linear pieces in
 * the coordinate of the 32-bit draw that places beta in the interval.  No
 * reference counterpart. */
#define NCGB_LP_K 126
#define NCGB_LP_NKNOTS 62   /* network quantile knots per egrid point */
typedef struct {
  double c1;        /* probability of the special first beta bin (0 if none) */
  uint32_t c1_thr;  /* the first bin is taken when a 32-bit draw is below this */
  float accept;     /* expected acceptance of the envelope */
  int32_t enabled;  /* 0: the plain percentile inversion is used */
  int32_t pad;
} ncgb_lp_hdr;
typedef struct {
  float aprob;      /* alias table: probability of keeping slot k */
  int32_t alias;    /* alias table: the other interval of slot k */
} ncgb_lp_slot;
typedef struct {
  double q;         /* interval k: beta = q + (2w+1) h for a 32-bit draw w */
  double h;         /* (interval width) * 2^-33 */
  float env;        /* envelope height on interval k */
  int32_t seg_lo;   /* its linear pieces: lp_seg[seg_lo .. seg_lo + seg_n) */
  int32_t seg_n;
  int32_t pad;
} ncgb_lp_cell;
typedef struct {
  uint32_t w0;      /* first draw w of the piece (beta(w0) >= bx[bin]) */
  float y0;         /* density at w0 */
  float slope;      /* density change per unit of w */
  int32_t bin;      /* the sampler's beta bin of the piece */
} ncgb_lp_seg;

/* One alpha cell [alpha_i, alpha_i+1] of a beta row: the constants of the
 * log-linear in-cell inversion (NCSABUtils.hh:282-304) for the middle part of
 * the alpha sampler: inv_bin = 1/(cumul_i+1 - cumul_i), ratio = S_i+1/S_i - 1,
 * slope = (alpha_i+1 - alpha_i)/(logS_i+1 - logS_i); slope is NaN where the
 * reference takes one of its degenerate branches. */
typedef struct {
  double inv_bin, ratio, slope, pad;
} ncgb_alpha_cell;

typedef struct {
  int64_t n;                 /* number of merged d-spacings */
  double threshold;          /* = two_dE[0]: Bragg cut-off energy */
  const double* two_dE;      /* ascending wl2ekin(2d) */
  const double* fdm_commul;  /* cumulative d*|F|^2*mult*xsectfact */
} ncgb_bragg_view;

typedef struct {
  int32_t n;
  double msd[NCGB_MAX_ELINC];
  double sigma[NCGB_MAX_ELINC]; /* bound incoherent xs * scale */
  float msd_f[NCGB_MAX_ELINC];  /* FP32 copies (mixed-precision mode) */
  float sigma_f[NCGB_MAX_ELINC];
} ncgb_elinc_view;

typedef struct {
  /* scalars */
  double kT, egrid_margin, internal_scale;
  double kext;          /* SABXSProvider: (xs(Emax)-extenderxs(Emax))*Emax */
  double k1, k2;        /* SABSampler: xsAtEmax*Emax, extenderxs(Emax)*Emax */
  double ext_sigma_free, ext_ca; /* free-gas extender, xs = sf*shape(ca*E) */
  double ext_kT, ext_mass_amu;
  double sigma_bound;
  int32_t ne, na, nb;
  float internal_scale_f; /* FP32 copy of internal_scale (mixed-precision mode) */
  /* energy grid */
  const double* egrid;  /* [ne] */
  const double* xs;     /* [ne] */
  const float* egrid_f; /* [ne] FP32 copy (mixed-precision mode) */
  const float* xsf;     /* [2*ne] (xs_i, (xs_i+1 - xs_i)/(egrid_i+1 - egrid_i)) in FP32 */
  /* energy-grid bucket index: for key k = (bits of E) >> 49 (f64) or >> 20
   * (f32) -- eight buckets per octave -- ebkt[k - kmin] is the first grid index
   * whose key is >= k (nbkt + 1 entries, the last = ne) */
  const int32_t* ebkt;
  const int32_t* ebkt_f;
  int64_t ebkt_kmin;
  int32_t ebkt_f_kmin;
  int32_t ebkt_n, ebkt_f_n;
  int32_t pad1;
  /* kernel grid, S stored beta-major: idx = ibeta*na + ialpha */
  const double* alpha;  /* [na] */
  const double* beta;   /* [nb] */
  const double* sab;    /* [nb*na] */
  const double* logsab; /* [nb*na] */
  const double* cumul;  /* [nb*na] cumulative alpha integrals per beta row */
  /* per energy-grid point sampler (kind 0: no scatter, 1: Alg.1) */
  const int32_t* smp_kind;        /* [ne] */
  const int32_t* smp_ibetaoffset; /* [ne] */
  const int32_t* smp_nbeta;       /* [ne] beta points in the sampler */
  const int64_t* smp_offset;      /* [ne] offset into bx/by/bcdf/info */
  const double* smp_fbkep;        /* [ne] first-bin kinematic endpoint (<=0) or 1.0 */
  const double* bx;               /* beta values */
  const double* by;               /* normalised pdf values */
  const double* bcdf;             /* normalised cdf values */
  const ncgb_alpha_info* info;    /* [offset + j], j < nbeta-1 */
  /* precomputed for the GPU (derived from the arrays above) */
  double inv_kT;
  const double* inv_dE;           /* [ne] 1/(egrid[i+1]-egrid[i]) */
  const double* inv_dbeta;        /* [nb] 1/(beta[i+1]-beta[i]) */
  const ncgb_beta_bin* bbin;      /* [offset + j]: bin j of a sampler, j < nbeta-1 */
  const ncgb_alpha_cell* acell;   /* [nb*na] */
  /* FP32 copies for the mixed-precision mode's alpha sampling */
  const float* alpha_f;           /* [na] */
  const float* sab_f;             /* [nb*na] */
  const float* logsab_f;          /* [nb*na] */
  const float* cumul_f;           /* [nb*na] */
  const float* acell_f;           /* [nb*na*4]: inv_bin, ratio, slope (NaN: degenerate), 0 */
  const float* inv_dbeta_f;       /* [nb] */
  const ncgb_alpha_info_f* info_f; /* indexed like info */
  /* learned beta proposal (NULL: none attached): lp_hdr[ne], lp_slot[ne*NCGB_LP_K],
   * lp_cell[ne*NCGB_LP_K], lp_seg[...] */
  const ncgb_lp_hdr* lp_hdr;
  const ncgb_lp_slot* lp_slot;
  const ncgb_lp_cell* lp_cell;
  const ncgb_lp_seg* lp_seg;
} ncgb_sab_view;

typedef struct {
  double kT, mass_amu, sigma_free, ca;
} ncgb_freegas_view;

typedef struct {
  int32_t type;
  float scale_f;               /* FP32 copy of scale (mixed-precision mode) */
  double scale, elow, ehigh;
  ncgb_bragg_view bragg;
  ncgb_elinc_view elinc;
  ncgb_sab_view sab;
  ncgb_freegas_view fg;
} ncgb_comp_view;

typedef struct {
  int32_t ncomp;
  int32_t pad0;
  double dom_elow, dom_ehigh; /* union of the component domains */
  ncgb_comp_view comp[NCGB_MAX_COMP];
  /* erfc at the 1101 bin edges of [-2,9] plus +-infinity, for the free-gas
   * sampler's cheap bounds (NCFreeGasUtils.cc:95-147); 1103 values */
  const double* fg_erfc_table;
  /* absorption (AbsOOV, NCAbsOOV.cc:33-44): xs = abs_c / sqrt(E); abs_c < 0:
   * not in the bundle */
  double abs_c;
} ncgb_material_view;

#ifdef __cplusplus
}
#endif

#endif
