/*
 * jld.h — C ABI of the GB300 (sm_103a) Lagrangian-Deep-Learning hot path.
 *
 * These entry points replace the XLA CPU custom-call targets that the
 * reference registers in lib/cpu.cc:271-292 (ppaint_*, preadout_*,
 * ppaint3D_*, preadout3D_*, buildplan_*, pfft_*, pifft_*, initLayout,
 * clean_*) for a world size of one.  Differences from the reference ABI:
 *
 *  - Every call is stream-ordered: it takes the cudaStream_t to launch on
 *    and device pointers to caller-owned buffers.  Nothing is allocated on a
 *    compute call; FFT twiddle tables are built once per (shape, dtype, device)
 *    by jld_buildplan_* (or lazily by the first FFT call, which must then
 *    happen outside stream capture).
 *  - Every call returns an int status (JLD_OK or a JLD_ERR_* code) and sets
 *    a thread-local message readable with jld_last_error().  The reference's
 *    custom calls return void (lib/cpu.cc:52) and throw from inside
 *    (lib/parops_fast.h:186).
 *  - The readouts are stateless: they use the positions passed to them,
 *    where the reference reads positions stored by the previous ppaint
 *    (lib/cpu.cc:93,137; lib/parops_fast.h:534-561).
 *  - The MPI communicator, layout index and edge arrays disappear: at world
 *    size one the decomposition of lib/parops_fast.h:52-161 keeps every
 *    particle on the local rank in input order, and the edges cover the whole
 *    mesh.
 *
 * Positions "in mesh units" are what the reference's custom calls receive
 * after jaxpops_bind.py:163-164 (pos % BoxSize, then / (BoxSize/Nmesh)),
 * flattened row-major as (N, 3).  The *_box entry points take positions in
 * box units and apply that same prelude on the device.
 *
 * Meshes are row-major (Nx, Ny, Nz), z fastest.  Half spectra are row-major
 * (Nx, Ny, Nz/2+1) — split into real and imaginary planes for the
 * reference-shaped pfft/pifft (lib/cpu.cc:169-245), interleaved complex for
 * the *_c variants.  Nz must be even.
 */
#ifndef JLD_H_
#define JLD_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define JLD_API __attribute__((visibility("default")))
#else
#define JLD_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* jld_stream_t; /* == cudaStream_t */

enum {
  JLD_OK = 0,
  JLD_ERR_ARG = 1,         /* null pointer, negative count, bad flag value */
  JLD_ERR_UNSUPPORTED = 2, /* mesh size the FFT does not factor (2,3,5), odd Nz */
  JLD_ERR_WORKSPACE = 3,   /* workspace pointer null or smaller than required */
  JLD_ERR_CUDA = 4,        /* a CUDA runtime call failed; see jld_last_error() */
  JLD_ERR_TIMEOUT = 5,     /* a bounded device wait gave up */
  JLD_ERR_NOPLAN = 6       /* FFT plan missing while the stream is capturing */
};

/* Library identity and error reporting (no reference counterpart). */
JLD_API const char* jld_version(void);
JLD_API const char* jld_status_string(int status);
JLD_API const char* jld_last_error(void);
/* Copies `bytes` from page-locked host memory to device memory with a  */
/* kernel that reads the host buffer directly (over NVLink-C2C on a GB300 */
/* node) instead of the copy engines; `ctas` CTAs of 1024 threads (<= 0: */
/* four), each holding an SM.  Both pointers 16-byte aligned.             */
/* Stream-ordered.  No counterpart in the reference (host-feed helper).   */
JLD_API int jld_copy_from_host(jld_stream_t stream, void* dst, const void* src_host, size_t bytes,
                               int32_t ctas);
/* Number of kernel nodes in a captured CUDA graph (cudaGraph_t passed as */
/* void*): the kernel launches one replay issues.  No counterpart in the  */
/* reference (measurement helper).                                        */
JLD_API int jld_graph_kernel_nodes(void* graph, int64_t* kernels);

/* ------------------------------------------------------------------ */
/* Layout bookkeeping.                                                  */
/* initLayout (lib/cpu.cc:29-38, lib/parops_fast.h:35-41) and clean_f32 / */
/* clean_f64 (lib/cpu.cc:40-49, lib/parops_fast.h:43-48).  Stateless      */
/* here: both validate lyidx (0..4, jaxpops_bind.py:157) and return.      */
JLD_API int jld_init_layout(int32_t commsize, int32_t lyidx);
JLD_API int jld_clean(int32_t lyidx);

/* ------------------------------------------------------------------ */
/* CIC paint.  ppaint_f32 / ppaint_f64: lib/cpu.cc:51-72 ->            */
/* lib/parops_fast.h:484-531 (lpaint 354-411).  out is overwritten     */
/* (zeroed, then painted).  mass has nparts entries.                   */
JLD_API int jld_ppaint_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                   const float* mass, int32_t nx, int32_t ny, int32_t nz,
                   float* out);
JLD_API int jld_ppaint_f64(jld_stream_t stream, const double* pos, int64_t nparts,
                   const double* mass, int64_t nx, int64_t ny, int64_t nz,
                   double* out);

/* Same paint on box-unit positions with the jaxpops_bind.py:161-164    */
/* prelude fused (mass broadcast, pos % box, / (box/N)).  mass may be   */
/* NULL, in which case every particle weighs mass_scalar.              */
JLD_API int jld_ppaint_box_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                       const float* mass, float mass_scalar,
                       int32_t nx, int32_t ny, int32_t nz, const float box[3],
                       float* out);
JLD_API int jld_ppaint_box_f64(jld_stream_t stream, const double* pos, int64_t nparts,
                       const double* mass, double mass_scalar,
                       int64_t nx, int64_t ny, int64_t nz, const double box[3],
                       double* out);

/* Accumulating box-unit paint: jld_ppaint_box_f32 without clearing `out` */
/* first, so that particles arriving in chunks (snapshot ingestion,       */
/* JERALD/snaputils.py:385-387 over a whole snapshot) add into one map.   */
JLD_API int jld_ppaint_box_acc_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                           const float* mass, float mass_scalar,
                           int32_t nx, int32_t ny, int32_t nz,
                           const float box[3], float* out);

/* Paint variants of the same box-unit paint (no reference counterpart;  */
/* same contract and results within float rounding):                    */
/*   method 0 = plain atomics, 1 = warp-aggregated atomics.             */
JLD_API int jld_ppaint_box_method_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                              const float* mass, float mass_scalar,
                              int32_t nx, int32_t ny, int32_t nz,
                              const float box[3], int32_t method, float* out);

/* Sort by cell key (no counterpart in the reference, whose decomposition */
/* computes the same key per particle, lib/parops_fast.h:91-93, but keeps  */
/* input order).  Box-unit positions, the jaxpops_bind.py:161-164 prelude  */
/* applied; keys[i] = the i-th smallest key, order[i] = its particle index, */
/* ties in input order (numpy.argsort(keys, kind="stable")).  A stable LSD  */
/* radix sort: workspace jld_cell_sort_workspace(nparts) bytes, 256-byte   */
/* aligned; nparts < 2^31 - 1, Nx*Ny*Nz < 2^31.                            */
JLD_API size_t jld_cell_sort_workspace(int64_t nparts);
JLD_API int jld_cell_sort_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                              int32_t nx, int32_t ny, int32_t nz, const float box[3],
                              int32_t* keys, int32_t* order, void* ws, size_t ws_bytes);
/* Paint of box-unit positions that walks a cell-key order from           */
/* jld_cell_sort_f32 (replaces lpaint, lib/parops_fast.h:354-411, with the */
/* same mesh): per run of equal keys (the particles of one cell) the eight */
/* corner weights are summed first -- runs longer than a warp's round of  */
/* 32 in FP64, rounded once -- and added to `out` (zeroed first) once per  */
/* corner.  The same order serves repeated paints of the same positions,  */
/* as the reference's stored layout does (useLayout,                      */
/* lib/parops_fast.h:484-531).                                             */
JLD_API int jld_ppaint_sorted_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                                  const float* mass, float mass_scalar, int32_t nx, int32_t ny,
                                  int32_t nz, const float box[3], const int32_t* keys,
                                  const int32_t* order, float* out);
/* jld_cell_sort_f32 then jld_ppaint_sorted_f32 in one call; workspace     */
/* jld_ppaint_box_sorted_workspace(nparts) bytes, 256-byte aligned.        */
JLD_API size_t jld_ppaint_box_sorted_workspace(int64_t nparts);
JLD_API int jld_ppaint_box_sorted_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                                      const float* mass, float mass_scalar, int32_t nx, int32_t ny,
                                      int32_t nz, const float box[3], float* out, void* ws,
                                      size_t ws_bytes);

/* Cell key of every particle: ((i % Nx) * Ny + j % Ny) * Nz + k % Nz with */
/* i = int(p_x) etc., the per-particle key of the reference's             */
/* decomposition (lib/parops_fast.h:91-93).  box == NULL: positions are in */
/* mesh units; otherwise box units with the jaxpops_bind.py:163-164        */
/* prelude applied.  keys has nparts int32 entries.                        */
JLD_API int jld_cell_keys_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                      int32_t nx, int32_t ny, int32_t nz, const float* box,
                      int32_t* keys);
JLD_API int jld_cell_keys_f64(jld_stream_t stream, const double* pos, int64_t nparts,
                      int64_t nx, int64_t ny, int64_t nz, const double* box,
                      int32_t* keys);

/* ------------------------------------------------------------------ */
/* CIC readout.  preadout_f32 / preadout_f64: lib/cpu.cc:74-94 ->       */
/* lib/parops_fast.h:533-567 (lreadout 414-481).  vjpdim = -1 reads the  */
/* field; vjpdim = d in {0,1,2} replaces the weight along d by its       */
/* derivative (+-Nmesh_d/box_d), as in lib/parops_fast.h:448-451.        */
JLD_API int jld_preadout_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                     const float* field, int32_t nx, int32_t ny, int32_t nz,
                     const float box[3], int32_t vjpdim, float* out);
JLD_API int jld_preadout_f64(jld_stream_t stream, const double* pos, int64_t nparts,
                     const double* field, int64_t nx, int64_t ny, int64_t nz,
                     const double box[3], int32_t vjpdim, double* out);
JLD_API int jld_preadout_box_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                         const float* field, int32_t nx, int32_t ny, int32_t nz,
                         const float box[3], int32_t vjpdim, float* out);
JLD_API int jld_preadout_box_f64(jld_stream_t stream, const double* pos, int64_t nparts,
                         const double* field, int64_t nx, int64_t ny, int64_t nz,
                         const double box[3], int32_t vjpdim, double* out);

/* ------------------------------------------------------------------ */
/* 3-channel paint.  ppaint3D_f32 / _f64: lib/cpu.cc:96-116 ->          */
/* lib/parops_fast.h:678-725 (lpaint3D 615-676).  mass is (nparts, 3)    */
/* row-major; out is (3, Nx, Ny, Nz).                                   */
JLD_API int jld_ppaint3d_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                     const float* mass, int32_t nx, int32_t ny, int32_t nz,
                     float* out);
JLD_API int jld_ppaint3d_f64(jld_stream_t stream, const double* pos, int64_t nparts,
                     const double* mass, int64_t nx, int64_t ny, int64_t nz,
                     double* out);
JLD_API int jld_ppaint3d_box_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                         const float* mass, int32_t nx, int32_t ny, int32_t nz,
                         const float box[3], float* out);
JLD_API int jld_ppaint3d_box_f64(jld_stream_t stream, const double* pos, int64_t nparts,
                         const double* mass, int64_t nx, int64_t ny, int64_t nz,
                         const double box[3], double* out);

/* ------------------------------------------------------------------ */
/* 3-channel readout.  preadout3D_f32 / _f64: lib/cpu.cc:118-138 ->      */
/* lib/parops_fast.h:823-857 (lreadout3D 729-821).  vjp = 0: field is    */
/* (3, Nx, Ny, Nz) and channel d is read into out[:, d]; vjp = 1: field  */
/* is one mesh and out[:, d] is its CIC-weight gradient along d.          */
JLD_API int jld_preadout3d_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                       const float* field, int32_t nx, int32_t ny, int32_t nz,
                       const float box[3], int32_t vjp, float* out);
JLD_API int jld_preadout3d_f64(jld_stream_t stream, const double* pos, int64_t nparts,
                       const double* field, int64_t nx, int64_t ny, int64_t nz,
                       const double box[3], int32_t vjp, double* out);
JLD_API int jld_preadout3d_box_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                           const float* field, int32_t nx, int32_t ny, int32_t nz,
                           const float box[3], int32_t vjp, float* out);
JLD_API int jld_preadout3d_box_f64(jld_stream_t stream, const double* pos, int64_t nparts,
                           const double* field, int64_t nx, int64_t ny, int64_t nz,
                           const double box[3], int32_t vjp, double* out);

/* ------------------------------------------------------------------ */
/* FFT plans.  buildplan_f32 / _f64: lib/cpu.cc:140-167 ->               */
/* lib/parfft.h:33-76.  Builds (once per device) the FP64-generated      */
/* twiddle tables for this shape and returns {localL, localstart} =      */
/* {Nx, 0}.  Call before any CUDA-graph capture that runs an FFT.        */
JLD_API int jld_buildplan_f32(int32_t nx, int32_t ny, int32_t nz, int32_t local_out[2]);
JLD_API int jld_buildplan_f64(int32_t nx, int32_t ny, int32_t nz, int32_t local_out[2]);

/* Workspace bytes the FFT entry points need (Nx*Ny*(Nz/2+1) complex).  */
/* Single-precision calls on power-of-two meshes (16 <= Nx, Ny, Nz/2 <=  */
/* 2048) run the TMA-pipelined passes when the input, workspace and       */
/* output are 16-byte aligned (8 for an interleaved r2c output), and the  */
/* generic passes otherwise; both give the same transform.                */
JLD_API size_t jld_fft_workspace_f32(int32_t nx, int32_t ny, int32_t nz);
JLD_API size_t jld_fft_workspace_f64(int32_t nx, int32_t ny, int32_t nz);

/* pfft_f32 / pfft_f64: lib/cpu.cc:169-200 -> lib/parfft.h:78-94,111-125. */
/* Unnormalised forward r2c DFT (sign -1); re/im are (Nx, Ny, Nz/2+1).    */
JLD_API int jld_pfft_f32(jld_stream_t stream, const float* data, int32_t nx, int32_t ny,
                 int32_t nz, float* re, float* im, void* ws, size_t ws_bytes);
JLD_API int jld_pfft_f64(jld_stream_t stream, const double* data, int32_t nx, int32_t ny,
                 int32_t nz, double* re, double* im, void* ws, size_t ws_bytes);
/* Interleaved-complex output variant of the same transform.              */
JLD_API int jld_pfft_c_f32(jld_stream_t stream, const float* data, int32_t nx, int32_t ny,
                   int32_t nz, void* out_c, void* ws, size_t ws_bytes);
JLD_API int jld_pfft_c_f64(jld_stream_t stream, const double* data, int32_t nx, int32_t ny,
                   int32_t nz, void* out_c, void* ws, size_t ws_bytes);

/* pifft_f32 / pifft_f64: lib/cpu.cc:202-245 -> lib/parfft.h:96-109,     */
/* 127-138.  Unnormalised inverse c2r DFT (sign +1): complex inverse     */
/* along x and y, then a c2r along z that ignores the imaginary parts of  */
/* kz = 0 and kz = Nz/2.                                                  */
JLD_API int jld_pifft_f32(jld_stream_t stream, const float* re, const float* im,
                  int32_t nx, int32_t ny, int32_t nz, float* out,
                  void* ws, size_t ws_bytes);
JLD_API int jld_pifft_f64(jld_stream_t stream, const double* re, const double* im,
                  int32_t nx, int32_t ny, int32_t nz, double* out,
                  void* ws, size_t ws_bytes);
JLD_API int jld_pifft_c_f32(jld_stream_t stream, const void* in_c, int32_t nx, int32_t ny,
                    int32_t nz, float* out, void* ws, size_t ws_bytes);
JLD_API int jld_pifft_c_f64(jld_stream_t stream, const void* in_c, int32_t nx, int32_t ny,
                    int32_t nz, double* out, void* ws, size_t ws_bytes);

/* Allocation-free variant of jld_pfft_c_f32 (no counterpart in the       */
/* reference).  For callers that cannot allocate device memory (a host     */
/* framework that owns all allocations, or a phase where allocating is not */
/* allowed): it takes no workspace and allocates nothing, keeping its      */
/* scratch and twiddle tables in fixed device arrays inside libjld (72 MiB */
/* of scratch, held by every GPU that loads the library until exit).       */
/* Limits: nx * ny * (nz/2 + 1) * 8 bytes <= 72 MiB (256^3 fits) and each */
/* size <= 4096; larger meshes return JLD_ERR_WORKSPACE / UNSUPPORTED.     */
/* The first call on a device resolves the arrays' addresses (make it      */
/* before any stream capture).  All calls share the arrays and rewrite    */
/* both (the twiddle table for their shape, the scratch by their passes): */
/* calls that overlap on the GPU race on either.                           */
JLD_API int jld_pfft_c_static_f32(jld_stream_t stream, const float* data, int32_t nx,
                                  int32_t ny, int32_t nz, void* out_c);

/* ------------------------------------------------------------------ */
/* Fused LDL step: forward of `nstep` displacement layers, final map and  */
/* loss, and the adjoint, in one stream-ordered call.  It computes what   */
/* the reference's model.py evaluates through jaxpops_bind (loss at        */
/* model.py:351-403, its gradient through value_and_grad at 410-413), for  */
/* kind 0 = "sm" (potential_gradient_sm, model.py:186-212, ReLU bias map   */
/* model.py:338-344) and kind 1 = "dm" (model.py:137-179, 346-347).        */
/* The workspace must be 256-byte aligned (cudaMalloc'd memory is).        */
/*   pos     (nparts, 3) float32 box-unit positions (device)               */
/*   params  device float32: 5 per layer (alpha, gamma, kh, kl, nu),      */
/*           then (mu, w, b) for kind 0                                    */
/*   target  (nx, ny, nz) device float32; mask the same or NULL            */
/*   L1      1: sum |F - target| (model default for "sm"), 0: squares      */
/*   grad_mode 0: the reference's VJP rules, 1: exact adjoint (differs    */
/*           from 0 only in d/d alpha)                                     */
/*   options bit 0: warp-aggregated paint atomics (else plain atomics);   */
/*           bit 1: generic pass kernels instead of the TMA-pipelined ones */
/*           bit 2: bin the particles into 16^3-cell tiles first (counting */
/*                  sort) and scatter through shared-memory tile windows   */
/*           bit 3: memory plan for large boxes: one force-mesh slot; the  */
/*                  adjoint recomputes the force meshes of layers          */
/*                  1 .. nstep-2 from their stored densities (one extra    */
/*                  spectral forward per such layer) instead of keeping    */
/*                  nstep-1 slots of 16 bytes per cell                      */
/*           schedule choices (same results, different speed):             */
/*           bit 4: x passes on radix-16 schedules where radix-8 ones fit  */
/*           bits 5-6: narrowest pipelined tile, 0 automatic, 1/2/3 =      */
/*                  4/8/16 columns                                         */
/*           bits 7-8: binning tile edge (bit 2), 0/1/2 = 16/8/20 cells    */
/*   out     device float64: [loss, d loss / d params ...]                 */
/* Call jld_ldl_prepare_f32 (or one eager step) before capturing the step */
/* into a CUDA graph; parameters are read from device memory, so a graph  */
/* replays with whatever `params` holds.                                  */
/* Error word of the pipelined single-precision FFT passes on the current */
/* device, read after a device synchronisation (0 = fine; nonzero = a pass */
/* gave up waiting for a tile copy and stopped early, so some output since */
/* the last reset is invalid); reset != 0 clears it.  No counterpart in    */
/* the reference.                                                          */
JLD_API int jld_fft_pipe_status(int32_t* value, int32_t reset);
/* Error-path check of the bounded device waits (no counterpart in the    */
/* reference, whose custom calls have no error channel: a `throw` inside  */
/* a void call, lib/parops_fast.h:186).  One CTA arms an mbarrier for a    */
/* copy that is never issued, polls it `polls` times (1 .. 2^22) with the  */
/* pipelined passes' bounded wait, gives up, writes 99 to `word` and       */
/* returns; no copy is in flight.  word == NULL: the pipelined FFT error   */
/* word (read it with jld_fft_pipe_status); otherwise a device int, e.g.   */
/* the fused step's word from jld_ldl_error_word_f32.                      */
JLD_API int jld_wait_selftest(jld_stream_t stream, int32_t polls, int32_t* word);
/* Workspace bytes for the given option bits (0 for invalid arguments);    */
/* jld_ldl_workspace_f32 is the size for options = 4, enough for any      */
/* option set without bit 3.  No counterpart in the reference (its        */
/* buffers are library globals, lib/cpu.cc:15-25).                        */
JLD_API size_t jld_ldl_workspace_f32(int32_t nx, int32_t ny, int32_t nz, int64_t nparts,
                                     int32_t nstep);
JLD_API size_t jld_ldl_workspace_opt_f32(int32_t nx, int32_t ny, int32_t nz, int64_t nparts,
                                         int32_t nstep, int32_t options);
JLD_API int jld_ldl_prepare_f32(int32_t nx, int32_t ny, int32_t nz, const float box[3]);
JLD_API int jld_ldl_step_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                             int32_t nx, int32_t ny, int32_t nz, const float box[3],
                             int32_t nstep, int32_t kind, int32_t L1, int32_t grad_mode,
                             int32_t options, const float* params, const float* target,
                             const float* mask, void* ws, size_t ws_bytes, double* out);
/* The rest of model.py's loss for the fused step (jld_ldl_step_ext_f32): */
/* the smoothing of the residual by |k|^-n + 1 (model.py:376-381), the map */
/* exponent and second field (model.py:357-361) and the validation loss   */
/* (model.py:416-465).  Mask, field2 and maskvalid are (Nx, Ny, Nz) float  */
/* meshes on the device.                                                  */
typedef struct jld_ldl_loss_ext {
  float n;                /* smoothing exponent; 0 = no smoothing          */
  float index;            /* F ** index; 1 = none                           */
  const float* field2;    /* F * field2, or NULL                            */
  const float* maskvalid; /* validation mask, or NULL (validation loss 0)   */
} jld_ldl_loss_ext;
/* jld_ldl_step_f32 with the loss options above; out holds one more value */
/* after the gradient: the validation loss (model.py:lossv).              */
JLD_API int jld_ldl_step_ext_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                                 int32_t nx, int32_t ny, int32_t nz, const float box[3],
                                 int32_t nstep, int32_t kind, int32_t L1, int32_t grad_mode,
                                 int32_t options, const float* params, const float* target,
                                 const float* mask, const jld_ldl_loss_ext* ext, void* ws,
                                 size_t ws_bytes, double* out);
/* The fused step for the "HI" kind (model.py:213-247 layers, 313-336      */
/* final map): each layer's potential adds the star-map source,            */
/*   potk = 1e-3 (a1 G1 r2c((rho+1e-8)^g1) + a2 G2 r2c(starmap^g2)),       */
/* and the map is ReLU(w ReLU(rho + zs)^mu - D + b) with the depletion     */
/* D = ReLU(beta1 c2r(r2c(starmap) Fk) + eta) + beta2 starmap^gamma3.      */
/*   params  10 per layer (a1, g1, kh1, kl1, nu1, a2, g2, kh2, kl2, nu2),  */
/*           then 12 (mu, w, b, beta1, khi, kli, nui, beta2, gamma3, xi,   */
/*           eta, zs)                                                       */
/*   starmap (nx, ny, nz) device float32 (starmap^e is taken as 0 where    */
/*           starmap <= 0, as are its derivatives)                          */
/* Other arguments and option bits as jld_ldl_step_f32.  The workspace    */
/* (jld_ldl_workspace_hi_f32) is jld_ldl_workspace_opt_f32's plus          */
/* nstep + 1 half spectra (8 (nz/2+1) nx ny bytes each) and two real       */
/* meshes.  No counterpart in the reference, which evaluates the HI model  */
/* through the primitives (jaxpops_bind) one operation at a time.          */
JLD_API size_t jld_ldl_workspace_hi_f32(int32_t nx, int32_t ny, int32_t nz, int64_t nparts,
                                        int32_t nstep, int32_t options);
JLD_API int jld_ldl_step_hi_f32(jld_stream_t stream, const float* pos, int64_t nparts,
                                int32_t nx, int32_t ny, int32_t nz, const float box[3],
                                int32_t nstep, int32_t L1, int32_t grad_mode, int32_t options,
                                const float* params, const float* target, const float* mask,
                                const float* starmap, void* ws, size_t ws_bytes, double* out);
/* Device pointer to the step's error word in `ws` (0 = fine; nonzero = a  */
/* pipelined pass gave up waiting for a tile copy and stopped early).      */
JLD_API int jld_ldl_error_word_f32(const void* ws, int32_t nx, int32_t ny, int32_t nz,
                                   int64_t nparts, int32_t nstep, const int** out);
/* Device pointer to the particle order of the last step run on `ws` with */
/* binning: entry s is the input index of the particle stored at s.        */
JLD_API int jld_ldl_order_f32(const void* ws, int32_t nx, int32_t ny, int32_t nz, int64_t nparts,
                              int32_t nstep, const int** out);
/* Device pointer to the positions after `layer` (1..nstep) layers of the */
/* last step run on `ws` (in the order of jld_ldl_order_f32 when binned).  */
JLD_API int jld_ldl_positions_f32(const void* ws, int32_t nx, int32_t ny, int32_t nz,
                                  int64_t nparts, int32_t nstep, int32_t layer,
                                  const float** out);

/* ------------------------------------------------------------------ */
/* Snapshot-map ingestion: the per-particle part of makemap              */
/* (JERALD/snaputils.py:253-406) for one chunk of snapshot particles.    */
/* pos_out = (pos / unit) % box (snaputils.py:379-380: float32 division, */
/* then the periodic wrap in float64, rounded to float32); for kind > 0, */
/* weights = the map kind's weight (snaputils.py:360-376) in float64,    */
/* rounded to float32.  Kinds: 0 dm (no weights), 1 Mstar, 2 ne, 3 nT,   */
/* 4 nHI, 5 neVz, 6 MstarVz, 7 XHI.  Fields a kind does not use may be    */
/* NULL; particle p's vz is vz[vz_stride * p] (vz_stride 3 and vz = the  */
/* Velocities array + 2 for (N, 3) velocities).                          */
/* c1 = 4.0475e-7 h^2 / a^3 XH / prod(box) * prod(Nmesh), c2 = 323.06014 */
/* (snaputils.py:351-355), sqrt_a = a^0.5.                               */
JLD_API int jld_snap_prep_f32(jld_stream_t stream, const float* pos, int64_t nparts, float unit,
                      const double box[3], int32_t kind, const float* masses,
                      const float* electron_abundance, const float* internal_energy,
                      const float* neutral_h_abundance, const float* vz, int64_t vz_stride,
                      double c1, double c2, double XH, double sqrt_a,
                      float* pos_out, float* weights);

#ifdef __cplusplus
}
#endif
#endif /* JLD_H_ */
