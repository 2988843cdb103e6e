/*
 * ncrystal_gb300.h -- C ABI of the GB300 batched non-oriented scattering path.
 *
 * Part 1 is a drop-in for the subset of NCrystal's C interface
 * (ncrystal_core/include/NCrystal/cinterface/ncrystal.h, NCrystal 4.4.2) that
 * a Monte Carlo code uses to evaluate non-oriented materials: the same symbol
 * names, handle types, argument meanings, error conventions and output
 * sentinels.  Linking this library instead of libNCrystal moves the
 * per-neutron work of the _many calls onto the GPU.
 *
 * Part 2 holds additions with no counterpart in the reference: FP32 and
 * device-pointer batch calls, the multi-material ragged batch, and a host-only
 * table loader used by tests.
 *
 * Materials: ncrystal_create_scatter() takes NCrystal cfg-strings.  The
 * host-side loading results for a cfg-string are read from a material bundle
 * (.ncgb) found in the directories of NCGB_BUNDLE_PATH (colon separated) or in
 * the package's bundles/ directory; bundles are written by ncgb_export, which
 * runs NCrystal's own material loading.  The tables are uploaded once to the
 * current CUDA device.
 *
 * Random numbers: every neutron of every call owns a Philox4x32-10 stream
 * (include/ncgb_philox.h).  Counter-based streams replace the reference's
 * sequential per-Scatter stream: results are reproducible for a given seed,
 * clone index and call sequence, independent of launch shape.
 *
 * Plain C: pointers and sizes only.
 */
#ifndef NCRYSTAL_GB300_H
#define NCRYSTAL_GB300_H

#include <stdint.h>
#include "ncgb_tables.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ===================== Part 1: NCrystal C interface subset ================ */

/* Handles (ncrystal.h:666-670).  Opaque; 'internal' points at a type-tagged
 * ref-counted object like the reference's (ncrystal.cc:166-182). */
typedef struct { void * internal; } ncrystal_process_t;
typedef struct { void * internal; } ncrystal_scatter_t;

/* Reference counting (ncrystal.h:672-676).  ncrystal_unref takes the ADDRESS
 * of a handle and invalidates it when the count reaches 0. */
int  ncrystal_refcount( void* object );
void ncrystal_ref( void* object );
void ncrystal_unref( void* object );
int  ncrystal_valid( void* object );
void ncrystal_invalidate( void* object );

/* Factories (ncrystal.h:699, :708, :718-731). */
ncrystal_scatter_t ncrystal_create_scatter( const char * cfgstr );
ncrystal_scatter_t ncrystal_create_scatter_builtinrng( const char * cfgstr, unsigned long seed );
ncrystal_scatter_t ncrystal_clone_scatter( ncrystal_scatter_t );
ncrystal_scatter_t ncrystal_clone_scatter_rngbyidx( ncrystal_scatter_t, unsigned long rngstreamidx );
ncrystal_scatter_t ncrystal_clone_scatter_rngforcurrentthread( ncrystal_scatter_t );

/* Casts (ncrystal.h:680-686). */
ncrystal_process_t ncrystal_cast_scat2proc( ncrystal_scatter_t );
ncrystal_scatter_t ncrystal_cast_proc2scat( ncrystal_process_t );

/* Process queries (ncrystal.h:759-775). */
const char * ncrystal_name( ncrystal_process_t );
int ncrystal_isnonoriented( ncrystal_process_t );
void ncrystal_domain( ncrystal_process_t, double* ekin_low, double* ekin_high );

/* Scalar evaluation (ncrystal.h:765-780). */
void ncrystal_crosssection_nonoriented( ncrystal_process_t, double ekin, double* result );
void ncrystal_samplescatterisotropic( ncrystal_scatter_t, double ekin,
                                      double* ekin_final, double* cos_scat_angle );
void ncrystal_genscatter_nonoriented( ncrystal_scatter_t, double ekin,
                                      double* result_angle, double* result_dekin );

/* Batched evaluation -- the GPU hot path.
 * ncrystal.h:1305-1309 / ncrystal.cc:1107-1141: results[repeat*n_ekin] (barn),
 *   -1.0 everywhere on error. */
void ncrystal_crosssection_nonoriented_many( ncrystal_process_t,
                                             const double * ekin,
                                             unsigned long n_ekin,
                                             unsigned long repeat,
                                             double* results );
/* ncrystal.h:1289-1294 / ncrystal.cc:1201-1245: index irepeat*n_ekin+i;
 *   E'=-1, mu=-999 everywhere on error. */
void ncrystal_samplescatterisotropic_many( ncrystal_scatter_t,
                                           const double * ekin,
                                           unsigned long n_ekin,
                                           unsigned long repeat,
                                           double* results_ekin,
                                           double* results_cos_scat_angle );
/* ncrystal.h:1355-1360 / ncrystal.cc:1301-1324 (obsolete in the reference,
 *   warns once): angle=acos(mu), dekin=E'-E; outputs untouched on error. */
void ncrystal_genscatter_nonoriented_many( ncrystal_scatter_t,
                                           const double * ekin,
                                           unsigned long n_ekin,
                                           unsigned long repeat,
                                           double* results_angle,
                                           double* results_dekin );

/* Absorption (ncrystal.h:669-700, ncrystal.cc:411-445, :1518-1571): the
 * standard factory's 1/v model AbsOOV (NCStdAbsFact.cc:49-52), xs =
 * c/sqrt(E) (NCAbsOOV.cc:33-44), evaluated on the GPU by
 * ncrystal_crosssection_nonoriented(_many) on the cast process. */
typedef struct { void * internal; } ncrystal_absorption_t;
ncrystal_absorption_t ncrystal_create_absorption( const char * cfgstr );
ncrystal_absorption_t ncrystal_clone_absorption( ncrystal_absorption_t );
ncrystal_process_t ncrystal_cast_abs2proc( ncrystal_absorption_t );
ncrystal_absorption_t ncrystal_cast_proc2abs( ncrystal_process_t );

/* Scatter with directions (ncrystal.h:782-786, ncrystal.cc:1159-1174 and
 * :1248-1282): for non-oriented materials, an isotropic scatter followed by an
 * outgoing direction at cosine mu to the incoming one with a uniform azimuth
 * (randNeutronDirectionGivenScatterMu, NCRandUtils.cc:51-96).  The _many form
 * repeats one energy and direction 'repeat' times.  On error: E' -1 and a
 * zero direction. */
void ncrystal_samplescatter( ncrystal_scatter_t, double ekin, const double (*direction)[3],
                             double* ekin_final, double (*direction_final)[3] );
void ncrystal_samplescatter_many( ncrystal_scatter_t, double ekin, const double (*direction)[3],
                                  unsigned long repeat, double* results_ekin, double* results_dirx,
                                  double* results_diry, double* results_dirz );

/* Error handling (ncrystal.h:1031-1051; ncrystal.cc:281-322).  As in the
 * reference, an error prints its message and calls exit(1) unless
 * ncrystal_sethaltonerror(0) was called first. */
int ncrystal_sethaltonerror( int );
int ncrystal_setquietonerror( int );
int ncrystal_error( void );
const char * ncrystal_lasterror( void );
const char * ncrystal_lasterrortype( void );
void ncrystal_clearerror( void );
void ncrystal_seterrhandler( void (*handler)(char*,char*) );

/* Version (ncrystal.h:1229-1230): the NCrystal version whose behaviour the
 * path reproduces. */
int ncrystal_version( void );
const char * ncrystal_version_str( void );

/* ===================== Part 2: additions (no reference counterpart) ======= */

/* Per-neutron status codes written by the kernels. */
#define NCGB_ST_OK 0
#define NCGB_ST_LOOPCAP 1      /* rejection loop cap hit (reference: CalcError) */
#define NCGB_ST_UNSUPPORTED 2  /* reserved (no kernel writes it) */
#define NCGB_ST_CALCERROR 3    /* E*E' == 0 in the (alpha,beta) -> mu conversion
                                  (reference: CalcError, NCKinUtils.cc:40-45) */

/* Fused cross-section + one isotropic scatter per neutron on device memory:
 * d_ekin[n] -> d_xs[n], d_ekin_final[n], d_mu[n] (any output may be NULL),
 * d_status[n] optional.  Neutron i draws from stream (seed, i, callseq, clone
 * index) of the handle; the call sequence advances by one per call.  Runs on
 * 'stream' (a cudaStream_t, NULL = legacy default stream); asynchronous.
 * Returns 0, or non-zero after setting the error state. */
int ncgb_scatter_device( ncrystal_scatter_t, const double* d_ekin, unsigned long n,
                         double* d_xs, double* d_ekin_final, double* d_mu,
                         int32_t* d_status, void* stream );

/* The scatter batch with the material's absorption cross-section beside the
 * scattering one, in the same pass over the energies (an MC step needs both):
 * d_xs_abs[n] = c/sqrt(E) of the AbsOOV model; any output may be NULL. */
int ncgb_xs_abs_scatter_device( ncrystal_scatter_t, const double* d_ekin, unsigned long n, double* d_xs,
                                double* d_xs_abs, double* d_ekin_final, double* d_mu, int32_t* d_status,
                                void* stream );

/* Scatters with directions on device memory: d_ekin[n], d_dir[n][3] ->
 * d_ekin_final[n], d_dir_final[n][3] (d_status optional); neutron i uses
 * stream i as in ncgb_scatter_device, the direction's draws following the
 * scatter's.  Asynchronous on 'stream'. */
int ncgb_scatter_dir_device( ncrystal_scatter_t, const double* d_ekin, const double* d_dir, unsigned long n,
                             double* d_ekin_final, double* d_dir_final, int32_t* d_status, void* stream );

/* No counterpart in the reference.  Same as ncgb_scatter_device (FP64
 * arrays), but allocates nothing: its working memory is a fixed array inside
 * the library (16 B per neutron, at most NCGB_NOALLOC_MAX_NEUTRONS neutrons per
 * call; larger batches are refused with a BadInput error).  For callers that
 * must not allocate device memory while they run, e.g. a transport code living
 * in a framework that owns all device memory through its own pool, or one that
 * cannot take cudaMalloc's device-wide synchronisation inside its loop.  All
 * calls share that array: calls that overlap on the GPU race.  The first call
 * on a device looks up the array's address (do it before any stream capture)
 * and keeps it for the life of the device's primary context (do not call it
 * again after cudaDeviceReset); the device holding the material must be
 * current.  It computes in the handle's mode with the handle's sampler, like
 * ncgb_scatter_device, and an empty or refused call consumes no call sequence
 * number.  Phase timing (ncgb_phase_timing) never applies to its launches. */
#define NCGB_NOALLOC_MAX_NEUTRONS 1048576u
int ncgb_scatter_device_noalloc( ncrystal_scatter_t, const double* d_ekin, unsigned long n,
                                 double* d_xs, double* d_ekin_final, double* d_mu,
                                 int32_t* d_status, void* stream );

/* Measurement instrument (no counterpart in the reference): the same batch
 * as ncgb_scatter_device on FP64 device arrays (synchronous; on the library's
 * own stream), with the S(alpha,beta) pass replaced by a copy of it that reads
 * the SM clock at its phase boundaries.  cycles[0..NCGB_SAB_NPHASES) receive
 * the lanes' summed clock cycles per phase -- claiming a queued neutron and
 * setting up its sampler, the beta draw, the alpha draw from two rows, the
 * acceptance tests, the conversion to (E', mu) and its write, and lanes idle
 * at the end of the pass -- and cycles[NCGB_SAB_NPHASES] the number of Alg.1
 * attempts.  Neutrons on the rare list (free-gas components, energies above
 * a component's energy grid) are sampled after the clocked loop, unclocked.
 * The clock reads themselves cost registers, so the profiled pass
 * is slower than the product one; its shares are what it is for.  Returns 0,
 * or non-zero after setting the error state. */
#define NCGB_SAB_NPHASES 6
int ncgb_sab_phase_profile( ncrystal_scatter_t, const double* d_ekin, unsigned long n, double* d_xs,
                            double* d_ekin_final, double* d_mu, unsigned long long* cycles );

/* Same with FP32 energies in and FP32 results out; all arithmetic in the
 * kernel stays FP64. */
int ncgb_scatter_device_f32( ncrystal_scatter_t, const float* d_ekin, unsigned long n,
                             float* d_xs, float* d_ekin_final, float* d_mu,
                             int32_t* d_status, void* stream );

/* Host-pointer FP32 batch (H2D + kernel + D2H inside, synchronous). */
void ncgb_crosssection_nonoriented_many_f32( ncrystal_process_t, const float* ekin,
                                             unsigned long n_ekin, float* results );
void ncgb_samplescatterisotropic_many_f32( ncrystal_scatter_t, const float* ekin,
                                           unsigned long n_ekin, float* results_ekin,
                                           float* results_cos_scat_angle );

/* Arithmetic mode of a handle (or a batch).  NCGB_MODE_EXACT (the default)
 * computes in FP64 throughout and reproduces the reference's results.
 * NCGB_MODE_MIXED evaluates the incoherent-elastic exponentials (cross-section
 * and angle sampling) and the log-linear alpha inversion of the S(alpha,beta)
 * sampler in FP32; the beta-CDF inversion, Bragg sums, rejection tests and
 * kinematics stay FP64.  Mixed-mode cross-sections agree with the exact ones
 * to about 1e-7 relative; sampled alpha values move by about 1e-7 relative,
 * so a rejection decision or the choice of a table bin near its edge can
 * differ for a small fraction of neutrons (the sampled distributions are
 * unchanged).  New handles start in the mode named by the environment
 * variable NCGB_MODE ("exact" or "mixed"; unset = exact); clones inherit the
 * mode.  ncgb_set_mode returns 0, or non-zero after setting the error state;
 * ncgb_get_mode returns the mode, or -1 on error. */
#define NCGB_MODE_EXACT 0
#define NCGB_MODE_MIXED 1
int ncgb_set_mode( ncrystal_scatter_t, int mode );
int ncgb_get_mode( ncrystal_scatter_t );

/* Fused cross-section + scatter with HOST arrays: ekin[n] -> xs[n], E'[n],
 * mu[n] (any output may be NULL), FP64 or FP32.  Copies in, runs and copies
 * out in chunks on two streams so that transfers overlap the kernels (host
 * arrays in pinned memory make the copies asynchronous).  Neutron i uses
 * stream index i, like ncgb_scatter_device.  Synchronous; on error the outputs
 * hold the samplescatter sentinels (xs -1, E' -1, mu -999). */
void ncgb_xs_scatter_many( ncrystal_scatter_t, const double* ekin, unsigned long n,
                           double* xs, double* ekin_final, double* mu );
void ncgb_xs_scatter_many_f32( ncrystal_scatter_t, const float* ekin, unsigned long n,
                               float* xs, float* ekin_final, float* mu );

/* Number of neutrons whose status was not NCGB_ST_OK in the last _many call on
 * this thread. */
unsigned long ncgb_last_nfailed( void );

/* Host-only material tables (no GPU): load a bundle and build the flat tables
 * in host memory.  NULL on failure (ncgb_tables_lasterror() says why). */
void* ncgb_tables_load( const char* bundle_path );
const char* ncgb_tables_lasterror( void );
int ncgb_tables_view( void* tables, ncgb_material_view* out );
unsigned long ncgb_tables_bytes( void* tables );
void ncgb_tables_free( void* tables );
/* Test support: one named table array / scalar of component 'comp'. */
int ncgb_tables_array( void* tables, int comp, const char* name, const void** ptr, unsigned long* count );
int ncgb_tables_scalar( void* tables, int comp, const char* name, double* out );

/* Ragged multi-material batches (no reference counterpart): one launch pair
 * for neutrons of many materials.  d_offsets[nmat+1] (int64, device memory,
 * ascending, d_offsets[0] = 0, d_offsets[nmat] = n) gives each material's
 * neutrons [d_offsets[k], d_offsets[k+1]); neutron o of material k draws from
 * stream (seed_k, o - d_offsets[k], batch call sequence, clone index_k), so
 * a batch reproduces the single-material calls of fresh handles.  The
 * handles must live on one device and outlive nothing: the batch keeps their
 * tables alive itself. */
typedef struct { void * internal; } ncgb_batch_t;
ncgb_batch_t ncgb_batch_create( const ncrystal_scatter_t* scatters, unsigned long nmat );
void ncgb_batch_destroy( ncgb_batch_t* );
int ncgb_batch_scatter_device( ncgb_batch_t, const double* d_ekin, const int64_t* d_offsets, unsigned long n,
                               double* d_xs, double* d_ekin_final, double* d_mu, int32_t* d_status,
                               void* stream );
/* Times the launch shapes (pick block 128/256/512 x S(alpha,beta) blocks per
 * SM x one or two lists in the S(alpha,beta) queue) on this batch's arrays and
 * keeps the fastest for the batch.  Two lists: free-gas neutrons and energies
 * above a component's energy grid on a list of their own, so that the other
 * neutrons' sampler has no call in its loop.  Results do not depend on the
 * shape. */
int ncgb_batch_autotune( ncgb_batch_t, const double* d_ekin, const int64_t* d_offsets, unsigned long n,
                         double* d_xs, double* d_ekin_final, double* d_mu, void* stream );
int ncgb_batch_config( ncgb_batch_t, int* pick_block, int* sab_blocks_per_sm );
/* 1 if the batch's S(alpha,beta) queue uses two lists, 0 for one (the
 * default before autotuning); the setter fixes it without autotuning. */
int ncgb_batch_split_lists( ncgb_batch_t, int* split_lists );
int ncgb_batch_set_split_lists( ncgb_batch_t, int split_lists );
/* Same as ncgb_batch_scatter_device, replayed as a CUDA graph (captured on
 * first use, updated in place afterwards). */
int ncgb_batch_graph_launch( ncgb_batch_t, const double* d_ekin, const int64_t* d_offsets, unsigned long n,
                             double* d_xs, double* d_ekin_final, double* d_mu, int32_t* d_status,
                             void* stream );
/* Arithmetic mode of the batch (NCGB_MODE_*; starts as NCGB_MODE below). */
int ncgb_batch_set_mode( ncgb_batch_t, int mode );
/* Host arrays: copies in, runs and copies out (synchronous). */
void ncgb_batch_xs_scatter_many( ncgb_batch_t, const double* ekin, const int64_t* offsets, unsigned long n,
                                 double* xs, double* ekin_final, double* mu );

/* ===================== Part 3: learned beta proposal (no reference counterpart)
 *
 * A small network (4 hidden layers of 128, BF16 tensor-core GEMMs with FP32
 * accumulation, trained on the GPU by this library's own forward and backward
 * kernels) predicts, from (log E, T), 62 quantile knots of the beta
 * distribution of an S(alpha,beta) component.  Attached to a component, the
 * knots of each sampler energy (egrid point) become a piecewise-constant
 * envelope over the sampler's own piecewise-linear beta density; beta is then
 * drawn by exact rejection from that envelope instead of by the percentile
 * inversion.  The sampled distribution is unchanged (the first beta bin's
 * special treatment and the alpha sampling stay as in the plain sampler);
 * egrid points outside the network's trained (E, T) range or with an envelope
 * acceptance below 'min_accept' keep the plain inversion. */
#define NCGB_SAMPLER_PLAIN 0
#define NCGB_SAMPLER_LEARNED 1
/* Which sampler a handle (or a batch) uses; clones inherit it.  LEARNED uses
 * the proposals attached to the handle's material, PLAIN ignores them. */
int ncgb_set_sampler( ncrystal_scatter_t, int sampler );
int ncgb_get_sampler( ncrystal_scatter_t );
int ncgb_batch_set_sampler( ncgb_batch_t, int sampler );

/* Composition of a handle's material: number of components, temperature (K),
 * and per component its type (NCGB_COMP_*), scale and egrid size (SAB). */
int ncgb_material_info( ncrystal_scatter_t, int* ncomp, double* temperature );
int ncgb_component_info( ncrystal_scatter_t, int comp, int* type, double* scale, unsigned long* ne );
int ncgb_sab_egrid( ncrystal_scatter_t, int comp, double* egrid_out );

/* (alpha, beta) sampled by S(alpha,beta) component 'comp' alone
 * (SABSampler::sampleAlphaBeta, NCSABSampler.cc:158-227) at d_ekin[n]; the
 * training set of the proposal.  Streams and call sequence as
 * ncgb_scatter_device; asynchronous on 'stream'. */
int ncgb_sab_sample_device( ncrystal_scatter_t, int comp, const double* d_ekin, unsigned long n,
                            double* d_alpha, double* d_beta, int32_t* d_status, void* stream );

typedef struct { void * internal; } ncgb_mlp_t;
/* Network on the current device, He-uniform initial weights from 'seed'. */
ncgb_mlp_t ncgb_mlp_create( unsigned long long seed );
void ncgb_mlp_destroy( ncgb_mlp_t* );
unsigned long ncgb_mlp_nparams( void );
/* FP32 master weights, flat: W_l [in][out] row-major then b_l, l = 0..4. */
int ncgb_mlp_get_params( ncgb_mlp_t, float* out );
int ncgb_mlp_set_params( ncgb_mlp_t, const float* in );
/* (E, T) range the inputs are normalised over and the network is valid in. */
int ncgb_mlp_set_ranges( ncgb_mlp_t, double emin, double emax, double tmin, double tmax );
/* Pinball loss and its gradient (flat layout, host array) on the first n
 * samples (device arrays: log E, T, asinh(beta)). */
int ncgb_mlp_gradients( ncgb_mlp_t, const float* d_loge, const float* d_temp, const float* d_target,
                        unsigned long n, float* h_grad, float* h_loss, void* stream );
/* Adam training: 'steps' batches drawn with replacement from n samples; the
 * mean loss of every 'trace_every' steps is written to h_trace (optional). */
int ncgb_mlp_train( ncgb_mlp_t, const float* d_loge, const float* d_temp, const float* d_target,
                    unsigned long n, unsigned long steps, unsigned int batch, float lr, unsigned long long seed,
                    float* h_trace, unsigned long trace_every, void* stream );
/* Knots (62 asinh(beta) values per point) at n points. */
int ncgb_mlp_knots( ncgb_mlp_t, const float* d_loge, const float* d_temp, unsigned long n, float* d_knots,
                    void* stream );
/* Attach the network's proposal to SAB component 'comp' of the handle's
 * material (shared by all handles of that material; batches copy the
 * material's tables when created).  mean_accept: mean envelope acceptance of
 * the enabled egrid points. */
int ncgb_attach_proposal( ncrystal_scatter_t, int comp, ncgb_mlp_t, double min_accept, double* mean_accept );
/* Same from explicit knots[ne*62] (host, asinh(beta)), e.g. for comparisons. */
int ncgb_attach_proposal_knots( ncrystal_scatter_t, int comp, const float* knots, double min_accept,
                                double* mean_accept );
int ncgb_detach_proposal( ncrystal_scatter_t, int comp );
/* Per egrid point: envelope acceptance and whether the proposal is used. */
int ncgb_proposal_acceptance( ncrystal_scatter_t, int comp, float* accept, int32_t* enabled );
/* Host-only: the same tables from host material tables (ncgb_tables_load),
 * and tables for ncgb_tables_view to carry (the CPU oracle's input). */
int ncgb_tables_build_proposal( void* tables, int comp, const float* knots, const unsigned char* allowed,
                                double min_accept, void* hdr_out, void* slot_out, void* cell_out, void* seg_out,
                                unsigned long* nseg );
int ncgb_tables_set_proposal( void* tables, int comp, const void* hdr, const void* slot, const void* cell,
                              const void* seg, unsigned long nseg );

/* Material bundles.  ncrystal_create_scatter looks a cfg-string's bundle up
 * in NCGB_BUNDLE_PATH, NCGB_BUNDLE_CACHE and the package's bundles/
 * directory.  If there is none and an exporter library can be loaded
 * (NCGB_EXPORT_LIB, else libncgb_export.so beside this library; it links the
 * NCrystal library, whose host-side material loading -- NCMAT parsing, hkl
 * planes, VDOS expansion, energy grids -- it runs in-process, the way
 * ncrystal_create_scatter does at ncrystal.cc:1510-1516), the bundle is
 * exported into the cache directory first, so any cfg-string NCrystal accepts
 * can be loaded.  Without an exporter a missing bundle is FileNotFound; a
 * cfg-string NCrystal rejects gives NCrystal's error.  (No counterpart in the
 * reference, which has no bundles.)
 *
 * ncgb_bundle_path writes the path of a cfg-string's bundle (exporting it if
 * need be) into out[outlen]; ncgb_bundle_cache_dir writes the directory
 * on-demand exports go to (NCGB_BUNDLE_CACHE, else the package's bundles/).
 * ncgb_create_scatter_bundle creates a scatter handle for the material of an
 * explicit bundle file (the NCrystal plugin's bundles carry no cfg-string).
 * All return 0 / a valid handle, or set the error state. */
int ncgb_bundle_path( const char* cfgstr, char* out, unsigned long outlen );
int ncgb_bundle_cache_dir( char* out, unsigned long outlen );
ncrystal_scatter_t ncgb_create_scatter_bundle( const char* bundle_path, unsigned long seed );

/* One isotropic scatter at energy ekin on the random stream of a caller's
 * 64-bit key (stream (key, 0, 0, the handle's stream index)), leaving the
 * handle's own call sequence alone: the scalar sampling of the NCrystal
 * plugin, whose key comes from NCrystal's RNG (ProcImpl::sampleScatterIsotropic,
 * NCProcImpl.hh:118-127, takes the caller's RNG).  Synchronous.  Returns 0, or
 * non-zero with the error state set and (E', mu) = (-1, -999). */
int ncgb_samplescatterisotropic_keyed( ncrystal_scatter_t, double ekin, unsigned long long key,
                                       double* ekin_final, double* mu );

/* Creates n scatter handles (the seed of ncrystal_create_scatter_builtinrng)
 * for materials given by cfg-strings, deriving the S(alpha,beta) samplers of
 * all of them in one batched device derivation (a temperature grid, a set of
 * crystals).  Materials already loaded on this device are reused.  Returns 0,
 * or 1 with the error state set and null handles. */
int ncgb_create_scatters( const char* const* cfgstrs, unsigned long n, unsigned long seed,
                          ncrystal_scatter_t* out );

/* Host and batched device derivation over all S(alpha,beta) components of
 * n bundles: the comparison of ncgb_sab_derive_compare summed over them, the
 * number of components, and the two total times in ms. */
int ncgb_sab_derive_compare_many( const char* const* bundle_paths, unsigned long n, double* max_rel_diff,
                                  long long* n_double_diff, long long* n_int_mismatch, long long* ncomp,
                                  double* ms_host, double* ms_device );

/* Device-side derivation of the S(alpha,beta) sampling tables (the
 * per-energy-point samplers of SABIntegrator::analyseEnergyPoint,
 * NCSABIntegrator.cc:283-309, :352-559): compares component 'comp' of a bundle
 * derived on the host and on the current CUDA device.  Integer arrays must
 * agree exactly (n_int_mismatch); doubles differ only where CUDA's log/exp
 * differ from the host's in the last place (n_double_diff, max_rel_diff).
 * Times in ms.  Material loading uses the device builder when the environment
 * sets NCGB_TABLES_BUILD=device. */
int ncgb_sab_derive_compare( const char* bundle_path, int comp, double* max_rel_diff, long long* n_double_diff,
                             long long* n_int_mismatch, double* ms_host, double* ms_device );

/* Phase timing for benchmarks: while enabled, every scatter batch records
 * CUDA events on its stream before and after its two kernels (the pick /
 * cross-section pass and the S(alpha,beta) pass).  ncgb_phase_times waits for
 * them, returns the summed milliseconds, the number of batches and the SAB
 * queue length of this thread's last batch, and forgets them. */
void ncgb_phase_timing( int enable );
int ncgb_phase_times( double* ms_pick, double* ms_sab, unsigned long* nbatches, unsigned long* last_nsab );

/* Bytes of device memory holding a handle's material tables. */
unsigned long ncgb_device_bytes( ncrystal_scatter_t );

/* ===================== Part 4: MiniMC on the device ==========================
 *
 * The reference's MiniMC (src/minimc: standard engine with forced collisions
 * and roulette, sphere/box/slab/cylinder geometries, constant/circular/
 * isotropic sources, standard histogram tallies) with the neutron population
 * resident in device memory and every collision done by this library's
 * scatter kernels.  Results are the reference's JSON document
 * (NCrystalMiniMCResults_v1), statistically equivalent (the random streams
 * differ); output.metadata.device adds the step count and device time. */

/* Replaces ncrystal_jsonquery (ncrystal.h:1244-1253, ncrystal.cc:2463-2473)
 * for the MiniMC queries, entries separated by the BEL character (0x07):
 *   ["mmc","run",CFGSTR,GEOMCFG,SRCCFG,ENGINECFG]
 *   ["mmc","run",CFGSTR,SCENARIO,ENGINECFG]
 *   ["mmc","scenario",CFGSTR,SCENARIO]
 *   ["mmc","inspectcfg","geom"|"src"|"engine",CFG]
 * (NCMMC_Query.cc:60-157).  Other queries are refused (BadInput).  Returns a
 * string to free with ncrystal_dealloc_string, or NULL on error. */
char* ncrystal_jsonquery( const char* query );
/* ncrystal.h:1219 */
void ncrystal_dealloc_string( char* );
/* The same run for an existing scatter handle (its mode, sampler and random
 * stream are used for the collisions; the material's absorption per the
 * engine's absorption option).  enginecfg may be NULL. */
char* ncgb_mmc_run( ncrystal_scatter_t, const char* geomcfg, const char* srccfg, const char* enginecfg );

#ifdef __cplusplus
}
#endif

#endif
