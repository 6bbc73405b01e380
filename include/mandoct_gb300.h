/*
 * mandoct_gb300.h -- C ABI of the GB300 (sm_103a) MandoCT reconstruction kernels.
 *
 * The reference (MandoCT-Taichi) has no native ABI: its hot path is Taichi kernels
 * that are methods of Python classes.  Each entry point below replaces one of those
 * kernels (cited per function as file:line in the reference).  The Python drop-in
 * (package reconstruction_program_taichi_gb300) binds this library with ctypes: each
 * function is looked up by name, given the argument types listed in its
 * declaration here, and called with raw device pointers taken from torch tensors.
 *
 * Conventions
 *   - Every pointer to bulk data is a DEVICE pointer owned by the caller.
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *   - Every function returns 0 (MCT_OK) or a negative MCT_E_* code and never
 *     synchronises the stream; mct_last_error_string() describes the last failure
 *     of the calling host thread.
 *   - No function allocates device memory; intermediate buffers are passed in and
 *     sized by the *_size queries.
 *   - Sinograms are [rows][views][cols] float32 unless stated otherwise, volumes
 *     are [z][y][x] float32 (the reference's array layouts).
 */
#ifndef MANDOCT_GB300_H
#define MANDOCT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCT_OK 0
#define MCT_E_INVALID (-1)     /* bad argument, size or geometry */
#define MCT_E_CUDA (-2)        /* CUDA runtime error (launch or device) */
#define MCT_E_UNSUPPORTED (-3) /* option not supported by this build */
#define MCT_E_TIMEOUT (-4)     /* a bounded device-side wait gave up */

/* geometry flags (mct_geom.flags) */
#define MCT_CONE 1        /* ConeBeam */
#define MCT_CURVED 2      /* CurvedDetector */
#define MCT_SHORT_SCAN 4  /* |TotalScanAngle| mod 360 >= 0.01 deg */
#define MCT_PMATRIX 8     /* PMatrixFile geometry */
#define MCT_ACCUMULATE 16 /* mct_fdk_bp adds to vol (view-chunked FBP); finish with mct_fdk_bp_finish */

/* storage types of packed / reduced-precision buffers */
#define MCT_F32 0
#define MCT_BF16 1
#define MCT_F16 2

/* Scan and image geometry; every field mirrors a member of the reference's
 * Mgfbp / Mgfpj / Mgfbp_ir objects (run_mgfbp.py:87-719, run_mgfpj_v2.py:113-214). */
typedef struct mct_geom {
    int32_t nu;          /* detector columns of this call (det_elem_count_horizontal[*oversample]) */
    int32_t nv;          /* detector rows of this call (det_elem_count_vertical_actual) */
    int32_t views;       /* view_num */
    int32_t nv_total;    /* det_elem_count_vertical (full detector) */
    int32_t row_begin;   /* det_elem_vertical_recon_range_begin */
    int32_t nx;          /* img_dim (square slices) */
    int32_t nz;          /* img_dim_z */
    int32_t flags;       /* MCT_CONE | MCT_CURVED | MCT_SHORT_SCAN | MCT_PMATRIX */
    int32_t view_mode;   /* recon_view_mode: 1 axial, 2 coronal, 3 sagittal */
    int32_t fp_steps;    /* ray-march step count K of the forward projector */
    float du, dv;        /* det_elem_width, det_elem_height [mm] */
    float u0, u_step;    /* array_u[0], array_u[1]-array_u[0] (backprojectors) */
    float v0, v_step;    /* array_v[0], array_v[1]-array_v[0] (backprojectors) */
    float px, pz;        /* img_pix_size, img_voxel_height [mm] */
    float cx, cy, cz;    /* img_center_x, img_center_y, img_center_z [mm] */
    float sid, sdd;      /* source_isocenter_dis, source_det_dis [mm] */
    float img_rot;       /* img_rot [rad] */
    float total_scan_angle; /* [rad] */
    float fp_step;       /* fpj_step_size, as a fraction of the voxel diagonal */
    float fp_z_per_view; /* helical gantry advance per view [mm] (0: circular) */
    int32_t view_begin;  /* scan index of this call's first view (view-chunked FBP; else 0) */
    int32_t views_total; /* views of the whole scan when chunked (0: equal to views) */
} mct_geom;

/* Per-view and per-element tables (DEVICE pointers, float32). */
typedef struct mct_tables {
    const float* angles;  /* [views]  array_angle (includes img_rot) */
    const float* u;       /* [nu]     array_u (forward projector) */
    const float* v;       /* [nv]     array_v (forward projector) */
    const float* cz;      /* [views]  per-view image centre z, or NULL for geom.cz */
    const float* pmatrix; /* [views*12] projection matrices (backprojectors), or NULL */
    const float* pmat_a;  /* [views*9]  matrix A = inv(P[:, :3]) (forward projector), or NULL */
    const float* pmat_xs; /* [views*3]  source positions (forward projector), or NULL */
} mct_tables;

/* ---------------------------------------------------------------- library */
const char* mct_version(void);
const char* mct_last_error_string(void);
/* Number of kernels this library has launched since load (all threads). */
uint64_t mct_launch_count(void);

/* ---------------------------------------------------------------- FBP / FDK */

/* Beam-hardening polynomial (optional) and cosine (+ Parker) weighting.
 * Replaces Mgfbp.BHCorrection run_mgfbp.py:946-954 and Mgfbp.WeightSgm :956-1011.
 * sgm element (row r, view j, col c) is read at sgm[r*row_stride + j*view_stride + c]
 * (sinogram files: row_stride = views*nu, view_stride = nu; post-log image stacks:
 * row_stride = nu, view_stride = nv*nu).  bh_coeffs is a device array of n_bh
 * coefficients or NULL.  weighted is [nv][views][nu]. */
int mct_weight(const mct_geom* g, const mct_tables* t, const float* sgm, int64_t row_stride,
               int64_t view_stride, const float* bh_coeffs, int32_t n_bh, float* weighted,
               void* stream);

/* Vertical Gaussian smoothing over +-10 rows (DetectorElementVerticalGaussFilterSize).
 * Replaces the first loop of Mgfbp.ConvolveSgmAndKernel run_mgfbp.py:1019-1029.
 * gauss_taps: [2*nv-1] device taps from GenerateGassianKernel. */
int mct_vgauss(const mct_geom* g, const float* weighted, const float* gauss_taps, float* out,
               void* stream);

/* Row convolution y[k] = du * sum_m x[m] h[k-m+nu-1] as a Toeplitz product, float32
 * SIMT path.  Replaces Mgfbp.ConvolveSgmAndKernel run_mgfbp.py:1030-1046.
 * weighted: [nv][views][nu]; taps: [2*nu-1]; filtered: VIEW-MAJOR [views][nv][nu]. */
int mct_filter(const mct_geom* g, const float* weighted, const float* taps, float* filtered,
               void* stream);

/* Tensor-core (tcgen05) variant of mct_filter: the float32 operands are split into
 * bf16 parts and the part products are accumulated in float32 tensor memory.
 * dtype MCT_F32: hi + mid + lo parts, the six products of total order <= 2 (the dropped
 * terms are ~2^-24 relative; ~1e-6 overall, the tensor pipe's float32 accumulation).
 * dtype MCT_BF16: hi + lo parts, A_hi B_hi + A_hi B_lo + A_lo B_hi (~1e-5 relative; up to
 * ~1e-4 on small detectors).
 * workspace: device buffer of mct_filter_tc_workspace_size(g, dtype) bytes, 1 KiB
 * aligned, holding the tiled operands; call mct_filter_tc_prepare once per filter taps
 * (it also clears the timeout flag), then mct_filter_tc per sinogram, with the same
 * dtype.  Replaces Mgfbp.ConvolveSgmAndKernel run_mgfbp.py:1030-1046.
 * mct_filter_tc_status synchronises the stream and returns MCT_E_TIMEOUT if a bounded
 * pipeline wait of an earlier launch gave up. */
size_t mct_filter_tc_workspace_size(const mct_geom* g, int32_t dtype);
int mct_filter_tc_prepare(const mct_geom* g, const float* taps, int32_t dtype, void* workspace, void* stream);
int mct_filter_tc(const mct_geom* g, const float* weighted, int32_t dtype, void* workspace, float* filtered,
                  void* stream);
int mct_filter_tc_status(const mct_geom* g, int32_t dtype, void* workspace, void* stream);

/* Weighting and the tensor-core row filter in one call: the sinogram (strides and
 * beam-hardening coefficients as mct_weight) is weighted element by element while it
 * is split into mct_filter_tc's bf16 operand parts, so the weighted float32 sinogram is
 * never written, then filtered into filtered [views][nv][nu] (workspace and dtype as
 * mct_filter_tc, prepared by mct_filter_tc_prepare).  Results equal mct_weight followed
 * by mct_filter_tc.  No vertical Gaussian: with one, call mct_weight, mct_vgauss and
 * mct_filter_tc.  Replaces BHCorrection + WeightSgm + ConvolveSgmAndKernel
 * (FilterSinogram) run_mgfbp.py:946-1046, 1282-1292. */
int mct_weight_filter(const mct_geom* g, const mct_tables* t, const float* sgm, int64_t row_stride,
                      int64_t view_stride, const float* bh_coeffs, int32_t n_bh, int32_t dtype, void* workspace,
                      float* filtered, void* stream);

/* Bytes of the packed backprojection operand for storage type dtype. */
size_t mct_packed_size(const mct_geom* g, int32_t dtype);

/* Pack a view-major filtered sinogram into the gather layout of mct_fdk_bp (buffer of
 * mct_packed_size bytes, 16-byte aligned).  Cone beam: per (view, row r < nv, column
 * c < nu-1) the bilinear coefficients {A, C-A, B-A, (D-C)-(B-A)} of the cell with
 * corners A = F[r][c], B = F[r][c+1], C = F[r+1][c], D = F[r+1][c+1]; row nv-1 is NaN
 * (an off-detector marker).  Fan beam: per (view, row, column c < nu-1) the pair
 * {A, B-A}.  dtype MCT_F32, MCT_BF16, or MCT_F16: float16 values are stored times a
 * power of two chosen from the input's largest magnitude (kept in the buffer's last
 * 16 bytes), so any float32 range packs without overflow; the backprojectors undo it. */
int mct_pack(const mct_geom* g, const float* filtered, void* packed, int32_t dtype, void* stream);

/* mct_pack for a source with any (row, view) element strides: element (view j, row r,
 * col c) is src[r*row_stride + j*view_stride + c] (a [nv][views][nu] sinogram has
 * row_stride = views*nu, view_stride = nu).  The packed layout is the same. */
int mct_pack_strided(const mct_geom* g, const float* src, int64_t row_stride, int64_t view_stride, void* packed,
                     int32_t dtype, void* stream);

/* Pixel-driven FDK / fan-beam backprojection of a packed filtered sinogram into
 * vol [nz][nx][nx] (overwritten).  Replaces Mgfbp.BackProjectionPixelDriven
 * run_mgfbp.py:1062-1187, including its rule that a voxel projecting outside the
 * detector in any view is zero. */
int mct_fdk_bp(const mct_geom* g, const mct_tables* t, const void* packed, int32_t dtype, float* vol,
               void* stream);

/* View-chunked FDK (Mgfbp_v2, run_mgfbp_v2.py:62-103, which backprojects view by view
 * to bound device memory): call mct_weight / mct_filter / mct_pack / mct_fdk_bp per
 * chunk of views with g->views = the chunk's views, g->view_begin = its first scan
 * view, g->views_total = the scan's views, the tables of the WHOLE scan, and (for the
 * backprojection) MCT_ACCUMULATE in g->flags on a volume zeroed before the first chunk.
 * A voxel that leaves the detector in any chunk is carried as NaN; this call, after
 * the last chunk, writes those voxels as 0 (SetTruncatedRegionToZero, :229-233). */
int mct_fdk_bp_finish(const mct_geom* g, float* vol, void* stream);

/* ---------------------------------------------------------------- helical FBP */

/* Helical rebinning parameters (Mgfbp_helical.__init__, run_mgfbp_helical.py:59-95). */
typedef struct mct_helical {
    int32_t nu;            /* detector columns */
    int32_t nv;            /* detector rows of the helical sinogram (det_elem_count_vertical) */
    int32_t views;         /* helical views (view_num before rebinning) */
    int32_t view_count;    /* views of each rebinned fan sinogram */
    int32_t n_slices;      /* reconstructed slices (len(array_z_pos)) */
    float dv;              /* det_elem_height [mm] */
    float sdd;             /* source_det_dis [mm] */
    float mag;             /* mag_ratio_isocenter = SDD / SID */
    float det_offset_vertical; /* [mm] */
    float dis_per_view;    /* table advance per view [mm] */
} mct_helical;

/* Rebin a helical sinogram sgm [nv][views][nu] into one fan sinogram per slice:
 * out [n_slices][view_count][nu], slice s at z = z_pos[s] (device array).  Replaces
 * Mgfbp_helical.SinogramRebinning run_mgfbp_helical.py:178-205 for all slices in one
 * launch: linear interpolation along the rows where the slice plane meets view
 * view_begin(s) + i, times SDD / sqrt(SDD^2 + v^2); 0 for views outside [0, views-2]. */
int mct_helical_rebin(const mct_helical* h, const float* sgm, const float* z_pos, float* out, void* stream);

/* ---------------------------------------------------------------- forward projection */

/* Bytes of the optional forward-projection workspace (gather copies of the volume:
 * cone beam, two float32 quad copies of 16 bytes per voxel; fan beam, one
 * x/y-transposed copy). */
size_t mct_fp_workspace_size(const mct_geom* g);

/* Ray-driven trilinear forward projection of vol [nz][nx][nx] for all views into
 * sgm [nv][views][nu] (overwritten).  Rays with mask != 1 (mask [nv][views][nu], or
 * NULL for none) give 0.  workspace (mct_fp_workspace_size bytes, 16-byte aligned, or
 * NULL) receives gather copies of vol: for cone beam, per voxel the z-pairs of the
 * voxel and of its neighbour along the copy's slow axis (16 bytes; a trilinear cell is
 * two adjacent elements) in [z][y][x] and [z][x][y] order, for fan beam an
 * x/y-transposed copy; views whose detector columns run along y read the transposed
 * order, so a warp's gathers are coalesced.  Results agree with and without the
 * workspace to float32 rounding (the same samples, so the same zero pattern).
 * Replaces
 * Mgfpj_v3.ForwardProjectionBilinear run_mgfpj_v3.py:184-366 and
 * Mgfbp_ir.ForwardProjectionBilinear run_mgfbp_iterative_recon_IRN_CGLS.py:494-676. */
int mct_fp(const mct_geom* g, const mct_tables* t, const float* vol, const float* mask, float* sgm,
           void* workspace, void* stream);

/* Bytes of the mct_fp_storage workspace for dtype (MCT_F32: mct_fp_workspace_size;
 * MCT_BF16 / MCT_F16: two 16-bit cell copies, 32 bytes per voxel (+16 for float16);
 * 0 if unsupported). */
size_t mct_fp_storage_workspace_size(const mct_geom* g, int32_t dtype);

/* mct_fp reading gather copies stored as dtype: MCT_F32 is mct_fp; MCT_BF16 or MCT_F16
 * (cone beam, workspace of mct_fp_storage_workspace_size bytes required) store every
 * voxel's whole 2x2x2 trilinear cell as 8 16-bit values, so a cell is one 16-byte
 * gather; the volume values are rounded to bf16 or (times a power of two chosen from
 * the volume's largest magnitude) to float16; interpolation and sums stay float32.
 * No counterpart in the reference (its projector is float32 only). */
int mct_fp_storage(const mct_geom* g, const mct_tables* t, const float* vol, const float* mask, float* sgm,
                   void* workspace, int32_t dtype, void* stream);

/* mct_fp_storage with a volume stored as vol_dtype: MCT_F32 is mct_fp_storage; MCT_BF16
 * (bf16 CG iterates; cone beam with a workspace) is read by the copy kernels only, so
 * the projector runs as for a float32 volume holding the same values.  No counterpart
 * in the reference (its iterates are float32). */
int mct_fp_storage_in(const mct_geom* g, const mct_tables* t, const void* vol, int32_t vol_dtype,
                      const float* mask, float* sgm, void* workspace, int32_t dtype, void* stream);

/* Exact transpose of mct_fp: vol += P^T sgm (vol is accumulated, not cleared).
 * No counterpart in the reference (its CGLS pairs mct_fp with the unmatched
 * backprojector below); used for matched-adjoint CGLS and autograd. */
int mct_fp_adjoint(const mct_geom* g, const mct_tables* t, const float* sgm, const float* mask,
                   float* vol, void* stream);

/* Bytes of the mct_fp_adjoint_cells workspace: 32 per voxel in cone beam (the 8
 * corner sums of each trilinear cell), 16 in fan beam (4 per slice cell). */
size_t mct_fp_adjoint_workspace_size(const mct_geom* g);

/* mct_fp_adjoint (vol += P^T sgm) with the scatter done in cell space: each ray
 * flushes a cell's corner sums with one (fan) or two (cone) 16-byte vector
 * reductions into workspace (mct_fp_adjoint_workspace_size bytes, 16-byte aligned,
 * cleared on the stream by this call), then one pass adds to each voxel the entries of
 * the cells that contain it.  Same operator as mct_fp_adjoint up to the order of the
 * float32 additions.  No counterpart in the reference. */
int mct_fp_adjoint_cells(const mct_geom* g, const mct_tables* t, const float* sgm, const float* mask,
                         float* vol, void* workspace, void* stream);

/* *count (device uint64) = number of trilinear samples of mct_fp whose stencil lies
 * inside the volume (rays with mask != 1 excluded): the forward projector's
 * algorithmic work.  No counterpart in the reference. */
int mct_fp_count_samples(const mct_geom* g, const mct_tables* t, const float* mask, uint64_t* count,
                         void* stream);

/* Effective ray map [nv][views][nu]: 0 where a sample inside the inscribed cylinder
 * leaves the volume through z, else 1.  Replaces
 * Mgfbp_ir.GenEffectiveMapForwardProjectionAgent
 * run_mgfbp_iterative_recon_IRN_CGLS.py:679-833. */
int mct_effective_map(const mct_geom* g, const mct_tables* t, float* mask, void* stream);

/* Oversample binning (mean of `bin` sub-columns) and optional noise:
 * in [nv][views][nu*bin] -> out [nv][views][nu]; photons > 0 adds
 * N0 e^{-p} + sqrt(.)*N(0,1) noise (clamped at 1e-6) then -log, with a counter-based
 * generator seeded by `seed`.  Replaces Mgfpj_v3.BinSinogram run_mgfpj_v3.py:368-375
 * and AddPossionNoise :381-391. */
int mct_bin_noise(const mct_geom* g, const float* in, int32_t bin, float photons, uint64_t seed,
                  float* out, void* stream);

/* ---------------------------------------------------------------- iterative reconstruction */

/* The reference CGLS "P^T": sum over views of a bilinear gather weighted by
 * distance_factor*pixel_size, then zero voxels whose u left the detector in any view.
 * sgm [nv][views][nu] (rows at mask==0 should already be zero); vol [nz][nx][nx]
 * overwritten.  Replaces Mgfbp_ir.BackProjectionPixelDrivenPerView
 * run_mgfbp_iterative_recon_IRN_CGLS.py:372-474 driven by :319-336 and
 * SetTruncatedRegionToZero :477-481. */
int mct_bp_ref_unmatched(const mct_geom* g, const mct_tables* t, const float* sgm, float* vol,
                         void* stream);

/* The same operator reading the sinogram as packed stencils (mct_pack_strided of the
 * [nv][views][nu] sinogram, dtype MCT_F32, MCT_BF16 or MCT_F16): one gather per voxel x view. */
int mct_bp_ref_unmatched_packed(const mct_geom* g, const mct_tables* t, const void* packed, int32_t dtype,
                                float* vol, void* stream);

/* ADMM-TV splitting step of run_mgfbp_iterative_recon_ADMM_CGLS.py:128-143, in place
 * on volume-sized vy, vx (split variables) and py, px (scaled duals): with the in-plane
 * forward differences D_y x, D_x x (0 at the far edge) and w = D x + p / rho, v = w
 * where |w| > threshold (else 0; the reference's rule is a hard threshold), then
 * p += rho * (D x - v).  No counterpart name in the reference (NumPy there). */
int mct_admm_shrink(const mct_geom* g, const float* x, float rho, float threshold, float* vy, float* vx, float* py,
                    float* px, void* stream);

/* Right-hand side of the ADMM x-step (FunctionY, :160-162): out = bpb + rho * (Dt vy + Dt vx)
 * - (Dt py + Dt px), Dt a [i] = a[i-1] - a[i] on interior indices, 0 at both ends. */
int mct_admm_rhs(const mct_geom* g, const float* bpb, const float* vy, const float* vx, const float* py,
                 const float* px, float rho, float* out, void* stream);

/* TV reweighting WR = 1/sqrt(|D x|^2 + beta) (forward differences, zero at the far
 * edge; z differences only when nz > 2).  Replaces Mgfbp_ir.GenerateWR
 * run_mgfbp_iterative_recon_IRN_CGLS.py:234-243.  x, wr: [nz][nx][nx]. */
int mct_tv_weights(const mct_geom* g, const float* x, float beta, float* wr, void* stream);

/* out = a*out_in + s * D^T W D x with interior-only backward differences
 * (a = 0 ignores out_in).  Replaces Mgfbp_ir.Dt_W_D
 * run_mgfbp_iterative_recon_IRN_CGLS.py:267-286. */
int mct_dtwd(const mct_geom* g, const float* x, const float* wr, float s, const float* out_in,
             float a, float* out, void* stream);

/* mct_dtwd fused with the CG step's inner product: out = a*out_in + s * D^T W D x and
 * *dot = sum x[i]*out[i] in float64 (device scalar, overwritten), in one pass over the
 * volume (out may be out_in).  Replaces the last Dt_W_D of the operator and the
 * np.sum(d * q) of TikhonovSol run_mgfbp_iterative_recon_IRN_CGLS.py:200-203.
 * partials: device scratch of mct_reduce_scratch_size() bytes. */
int mct_dtwd_dot(const mct_geom* g, const float* x, const float* wr, float s, const float* out_in,
                 float a, float* out, double* partials, double* dot, void* stream);

/* sum sqrt(|D x|^2 + beta) accumulated in float64 into *result (device, overwritten).
 * Replaces Mgfbp_ir.TVPenaltyVal run_mgfbp_iterative_recon_IRN_CGLS.py:245-254.
 * partials: device scratch of mct_reduce_scratch_size() bytes. */
int mct_tv_penalty(const mct_geom* g, const float* x, float beta, double* partials, double* result,
                   void* stream);

/* Scratch bytes needed by the float64 reductions below. */
size_t mct_reduce_scratch_size(void);

/* The operator application of one CG step with the vector work in the backprojector's
 * epilogue: q = P^T p + s1 * D^T W1 D d (+ s2 * D^T W2 D d when wr2 is given; no TV
 * term when wr1 is NULL), each term added to the running value in that order, and
 * *dq = sum d[i] * q[i] in float64 over the stored q (device scalar, overwritten), so
 * q is written once and never re-read.  p is the packed sinogram of
 * mct_bp_ref_unmatched_packed (dtype its storage type); d and q are volumes of
 * vec_dtype (MCT_F32 or MCT_BF16), wr1 / wr2 float32.  Axial view mode, cone beam.
 * partials: device scratch of mct_bp_cg_partials_size(g) bytes (one float64 per
 * block, summed in a fixed order).  Replaces, per CG iteration of TikhonovSol
 * (run_mgfbp_iterative_recon_IRN_CGLS.py:198-203; ..._piccs.py:120-125), the
 * BackProjection of ForwardProjectionAndBackProjection (:288-316, kernel :372-474),
 * the Dt_W_D terms (:267-286) and np.sum(d * q). */
size_t mct_bp_cg_partials_size(const mct_geom* g);
int mct_bp_ref_unmatched_packed_cg(const mct_geom* g, const mct_tables* t, const void* packed, int32_t dtype,
                                   const void* d, const float* wr1, float s1, const float* wr2, float s2, void* q,
                                   int32_t vec_dtype, double* partials, double* dq, void* stream);

/* *result = sum a[i]*b[i] in float64 (device scalar).  Replaces the np.sum inner
 * products of TikhonovSol run_mgfbp_iterative_recon_IRN_CGLS.py:202-203, 216. */
int mct_dot_f64(const float* a, const float* b, int64_t n, double* partials, double* result,
                void* stream);

/* The same float64 inner product for callers that cannot allocate device memory
 * (for example an application that manages all GPU memory itself and passes the
 * library only its input and output buffers).  No counterpart in the reference.
 * The per-block partial sums live in a fixed 512 KiB device array inside the
 * library, held by every GPU that loads it until the process exits, so
 * n <= 134,217,728; larger n returns MCT_E_INVALID.  The first call on a device
 * looks up that array's address (make it before any stream capture) and keeps it for
 * the process: it stays valid in the device's primary context (the runtime API's
 * context) until that context is destroyed, so after a cudaDeviceReset, or from
 * another context on the same device, use mct_dot_f64 instead.  All calls
 * share the array: calls that overlap on the GPU race and must be serialised by the
 * caller.  No cudaMalloc/cudaFree is made. */
int mct_dot_f64_noalloc(const float* a, const float* b, int64_t n, double* result, void* stream);

/* One fused CGLS step on device scalars (no host round trip), following
 * TikhonovSol run_mgfbp_iterative_recon_IRN_CGLS.py:198-217:
 *   alpha = rr / dq;  x += alpha d;  r -= alpha q;  rr_new = sum r^2 (float64);
 * rr and dq are device float64 scalars; rr_new receives sum r^2 of the updated r.
 * The second call, mct_cgls_direction, finishes beta = rr_new/rr and d = r + beta d. */
int mct_cgls_update(int64_t n, const double* rr, const double* dq, float* x, float* r,
                    const float* d, const float* q, double* partials, double* rr_new, void* stream);
int mct_cgls_direction(int64_t n, const double* rr, const double* rr_new, const float* r, float* d,
                       void* stream);

/* ---- the CG vector operations on float32 or bf16 volumes (bf16 iterate storage).
 * No counterpart in the reference (its iterates are float32 NumPy arrays).  Elements
 * are widened to float32 for the arithmetic, reductions accumulate in float64, and
 * stored results are rounded to the volume's type; the float64 sums use the stored
 * values (|r|^2 of the rounded r, <d, q> of the rounded q).  dtype, x_dtype, vec_dtype
 * and vol_dtype are MCT_F32 or MCT_BF16. */

/* mct_bp_ref_unmatched_packed writing vol as vol_dtype (MCT_BF16: axial view mode, cone
 * beam). */
int mct_bp_ref_unmatched_packed_out(const mct_geom* g, const mct_tables* t, const void* packed, int32_t dtype,
                                    void* vol, int32_t vol_dtype, void* stream);
/* mct_tv_weights of x stored as x_dtype (wr stays float32). */
int mct_tv_weights_t(const mct_geom* g, const void* x, int32_t x_dtype, float beta, float* wr, void* stream);
/* out = a*out_in + s * D^T W D x on vec_dtype volumes (wr float32); with partials and dot
 * (both or neither) also *dot = sum x[i]*out[i] in float64, as mct_dtwd_dot. */
int mct_dtwd_t(const mct_geom* g, const void* x, const float* wr, float s, const void* out_in, float a, void* out,
               int32_t vec_dtype, double* partials, double* dot, void* stream);
/* mct_dot_f64, mct_cgls_update and mct_cgls_direction on dtype volumes. */
int mct_dot_f64_t(const void* a, const void* b, int64_t n, int32_t dtype, double* partials, double* result,
                  void* stream);
int mct_cgls_update_t(int64_t n, int32_t dtype, const double* rr, const double* dq, void* x, void* r,
                      const void* d, const void* q, double* partials, double* rr_new, void* stream);
int mct_cgls_direction_t(int64_t n, int32_t dtype, const double* rr, const double* rr_new, const void* r, void* d,
                         void* stream);

/* ---------------------------------------------------------------- synthetic data */

/* Exact line integrals of ellipsoids for the forward projector's ray geometry
 * (no counterpart in the reference; it generates seeded phantoms for benchmarks).
 * ell: [n_ell][10] = {cx, cy, cz, ax, ay, az, phi, theta?, psi?, mu}: centre [mm],
 * semi-axes [mm], rotation about z [rad] (indices 7, 8 reserved = 0), attenuation
 * [1/mm].  sgm [nv][views][nu] overwritten. */
int mct_project_ellipsoids(const mct_geom* g, const mct_tables* t, const float* ell, int32_t n_ell,
                           float* sgm, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MANDOCT_GB300_H */
