/*
 * pq3d -- GB300 (sm_103a) kernels for the quasi-dynamic earthquake-cycle hot
 * path of PyQuake3D, behind a plain C ABI (no torch types, plain pointers).
 *
 * Two kinds of entry points:
 *   1. Drop-in replacements of the reference shared library TDstressFS_C.so
 *      (src/TDstressFS_C.cpp).  Same symbol names, argument meaning, host
 *      pointers, `void` return.  They run on the current CUDA device.  Errors
 *      are printed to stderr, recorded for pq3d_last_error() and the outputs
 *      are filled with NaN (the reference has no error channel).
 *   2. Device entry points (pq3d_*): device pointers, a cudaStream_t passed as
 *      void*, an int status (PQ3D_OK = 0) and pq3d_last_error() for the text.
 *
 * Layouts
 *   stress/strain: [n][6] row-major, order xx, yy, zz, xy, xz, yz.
 *   nodes: [Nn][3] metres; tris: [N][3] 1-based node ids (gmsh / readmsh).
 *   Dense traction operator K: (3N) x (2N) row-major.  Row 3i+c is traction
 *     component c (0: along e1, 1: along e2, 2: normal) at receiver i (the
 *     centroid of element i); column 2j+s is unit slip s (0: strike, 1: dip)
 *     on source element j.  The reference's six N x N matrices are the strided
 *     views A1s = K[3i+0][2j+0], A1d = K[3i+0][2j+1], A2s = K[3i+1][2j+0],
 *     A2d = K[3i+1][2j+1], Bs = K[3i+2][2j+0], Bd = K[3i+2][2j+1]
 *     (src/QDsim_gpu.py:1745-1878).
 */
#ifndef PQ3D_H
#define PQ3D_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PQ3D_OK 0
#define PQ3D_ERR_ARG 1          /* bad argument (null pointer, size, alignment) */
#define PQ3D_ERR_CUDA 2         /* a CUDA call failed */
#define PQ3D_ERR_TIMEOUT 3      /* a bounded device-side wait gave up */
#define PQ3D_ERR_STEP 4         /* dt < 1e-15 or more than 20 rejected attempts */
#define PQ3D_ERR_UNSUPPORTED 5  /* a feature the library does not provide */

/* Text of the last error raised on the calling host thread ("" if none). */
const char *pq3d_last_error(void);
/* ABI version of this library. */
int pq3d_version(void);

/* ---------------- drop-in: reference TDstressFS_C.so ---------------- */

/* Stress and strain at n receivers (X, Y, Z) from one triangle P1, P2, P3
 * (3 doubles each) with Burgers vector strike Ss, dip Ds, tensile Ts.
 * Replaces src/TDstressFS_C.cpp:2095-2152 (ctypes binding src/Hmatrix.py:32-46). */
void TDstressFS_C(const double *X, const double *Y, const double *Z, size_t n,
                  const double *P1, const double *P2, const double *P3,
                  double Ss, double Ds, double Ts, double mu, double lambda_,
                  bool jud_halfspace, double *stress, double *strain);

/* Stress and strain at one receiver (x, y, z) from n_sources triangles
 * (P*_flat: [n_sources][3]).  Outputs [n_sources][6].
 * Replaces src/TDstressFS_C.cpp:2155-2200 (ctypes binding src/Hmatrix.py:48-56). */
void TDstressEachSourceAtReceiver_C(double x, double y, double z,
                                    const double *P1_flat, const double *P2_flat, const double *P3_flat,
                                    size_t n_sources, double Ss, double Ds, double Ts,
                                    double mu, double lambda_, bool jud_halfspace,
                                    double *stress_out, double *strain_out);

/* Legacy full-space variant with twelve separate output arrays.
 * Replaces src/TDstressFS_C.cpp:570-609. */
void TDstressFS_C1(const double *X, const double *Y, const double *Z, size_t n,
                   const double *P1, const double *P2, const double *P3,
                   double Ss, double Ds, double Ts, double mu, double lambda_,
                   double *Sxx, double *Syy, double *Szz, double *Sxy, double *Sxz, double *Syz,
                   double *Exx, double *Eyy, double *Ezz, double *Exy, double *Exz, double *Eyz);

/* ---------------- device: Green's-function assembly ---------------- */

/* Bytes of device workspace pq3d_assemble_dense needs for N elements. */
size_t pq3d_gf_workspace_bytes(int64_t N);

/* Dense traction operator rows for receivers [row0, row1) against all N
 * sources, FP64 (K64, required) and FP32 (K32, may be NULL).  K64/K32 point at
 * row 3*row0 of the (3N) x (2N) layout above (leading dimension 2N).  Replaces
 * the dense assembly QDsim_gpu.get_coreAB_mulproess (src/QDsim_gpu.py:1787-1878)
 * and its per-column TDstressFS + GetTtstress (src/QDsim_gpu.py:1745-1785).
 * nodes, tris, K64, K32, workspace: device pointers (16-byte aligned). */
int pq3d_assemble_dense(const double *nodes, const int64_t *tris, int64_t N,
                        int64_t row0, int64_t row1, double mu, double lambda_, int halfspace,
                        double *K64, float *K32, void *workspace, size_t workspace_bytes,
                        void *stream);

/* Variant of pq3d_assemble_dense that allocates nothing and takes no
 * workspace -- no counterpart in the reference.  For callers that cannot call
 * cudaMalloc: a host application whose device memory is handed out by its own
 * pool allocator (for example a framework that reserves the device memory up
 * front and forbids side allocations), or a loop that cannot afford the
 * implicit device synchronisation and the failure modes of cudaMalloc/cudaFree
 * between its launches.  The source and receiver tables live in a fixed
 * 14.2 MB __device__ array inside this library, so N is limited to 32768
 * elements (larger N returns PQ3D_ERR_ARG).  Every call looks up the array's
 * device address with the calling device current (cudaGetSymbolAddress; no
 * cached address, so a device reset between calls is harmless); the first
 * call on a device may load the library's device code, so make it before any
 * stream capture.  All calls
 * share the one array: calls that overlap on the GPU (other streams, other host
 * threads) race on it, so serialise them.  The caller still provides nodes,
 * tris, K64 and K32 as in pq3d_assemble_dense. */
int pq3d_assemble_dense_noalloc(const double *nodes, const int64_t *tris, int64_t N, int64_t row0, int64_t row1,
                                double mu, double lambda_, int halfspace, double *K64, float *K32, void *stream);

/* Host-buffer variant for callers that keep the mesh and the operator in host
 * memory (the reference keeps A1s..Bd as NumPy arrays): copies the mesh in and
 * assembles.  Outputs in page-locked host memory mapped into the device address
 * space (cudaHostAlloc, cudaHostRegister) are written by the assembly kernel
 * directly; other (pageable) outputs are assembled in row blocks on two
 * streams, each block copied back while the next one is computed.
 * K64_host: (3N)x(2N) doubles; K32_host may be NULL.  Allocates and frees its
 * own device buffers. */
int pq3d_assemble_dense_host(const double *nodes_host, int64_t n_nodes, const int64_t *tris_host,
                             int64_t N, double mu, double lambda_, int halfspace,
                             double *K64_host, float *K32_host);

/* ---------------- device: dense stepping (plain FP64) ---------------- */

/* out[r] = sum_c K[r][c] * v[c] for the (3N) x (2N) FP64 operator: the traction
 * product K.(V - Vpl) of src/QDsim_gpu.py:948-957 (v interleaved [j][strike,dip]). */
int pq3d_dense_matvec_f64(const double *K64, int64_t N, const double *v, double *out, void *stream);
/* Same with the FP32 operator copy: compensated FP32 products and sums (the
 * FP32-rounded operator applied to v to ~2^-44 relative).  v is given split
 * into FP32 pieces, vsplit[j] = (hi_strike, hi_dip, lo_strike, lo_dip) with
 * v ~= hi + lo (16-byte aligned, N x 4 floats). */
int pq3d_dense_matvec_f32(const float *K32, int64_t N, const float *vsplit, double *out, void *stream);

/* Device-resident state of one dense simulation; every pointer is a device
 * array of N doubles unless stated.  Field meaning follows the reference
 * QDsim_gpu attributes (src/QDsim_gpu.py:893-940). */
typedef struct pq3d_dense_sim {
    int64_t N;
    /* state y = (sigma, tau1, tau2, psi), MPa / MPa / MPa / - */
    double *Tno, *Tt1o, *Tt2o, *state;
    /* slip rate, rake, slip, friction */
    double *slipv1, *slipv2, *slipv, *rake, *slip1, *slip2, *slip, *Tt, *fric;
    /* per-cell parameters */
    const double *a, *b, *dc, *f0, *shear_loading, *normal_loading, *rake0;
    /* traction rates out[3N] = K.(V-Vpl): [3i+0]=AdotV1, [3i+1]=AdotV2, [3i+2]=Bs.v1+Bd.v2 */
    double *rates;
    /* scratch: vprime[2N] (FP64 operator: v' as [N] double2; FP32 operator: its
     * hi/lo split as [N] float4), cand[4N] */
    double *vprime, *cand;
    /* FP64 operator (3N)x(2N) or FP32 operator (exactly one non-NULL) */
    const double *K64;
    const float *K32;
    /* device control block: see pq3d_step_ctrl */
    struct pq3d_step_ctrl *ctrl;
    /* scalars */
    double V0, Vpl, eta;   /* eta = mu / (2 cs) */
    int fix_Tn;
    /* Pore-pressure dilatancy (src/QDsim_gpu.py:611-671), all NULL when off:
     * P, dPdt [N] (Pa, Pa/s) enter the right-hand side; Parr [ndepth + 1][N]
     * is the fault-normal pressure profile of every cell (row k = depth node
     * k, the last row the fixed far-field value); dila = the table built by
     * pq3d_dilatancy_table.  After every accepted step each cell takes one
     * implicit diffusion step (tridiagonal, ndepth unknowns). */
    int32_t ndepth;
    double *P, *dPdt, *Parr;
    const double *dila;
} pq3d_dense_sim;

/* Dilatancy table for pq3d_dense_sim.dila from the depth nodes z[ndepth + 1]
 * (the reference's zp = log(1 + yp / 1e-2), yp logspace(-3, 10, 60)) and the
 * parameter-file values (hydraulic diffusivity c_hyd, dilatancy coefficient,
 * shear-zone thickness, effective compressibility, far-field pressure P0 in
 * Pa).  out[pq3d_dilatancy_table_len(ndepth)] (host memory). */
size_t pq3d_dilatancy_table_len(int ndepth);
int pq3d_dilatancy_table(const double *z, int ndepth, double c_hyd, double dilatancy, double thickness,
                         double compressibility, double P0, double *out);

/* Device control block of the stepper (one per simulation, device memory).
 * The host writes dttry/time/status before the first step; the stepper clears
 * the reduction and barrier fields itself at every launch. */
typedef struct pq3d_step_ctrl {
    double dttry;          /* in: first trial dt of the next step; out: dtnext */
    double time;           /* simulated time (s) */
    double maxv;           /* max |V| after the last accepted step */
    int32_t status;        /* PQ3D_OK or PQ3D_ERR_STEP / PQ3D_ERR_TIMEOUT */
    int32_t steps_done;    /* accepted steps since the control block was reset */
    int64_t attempts;      /* attempted steps (7 right-hand-side evaluations each) */
    uint64_t err_slot[6];  /* 3 rotating slots x (psi error, traction error), double bits */
    uint64_t maxv_bits;    /* max |V| reduction (double bits) */
    uint32_t bar_count;    /* grid barrier arrival counter */
    uint32_t bar_gen;      /* grid barrier generation */
} pq3d_step_ctrl;

/* Advance `nsteps` accepted steps on the device.  h_hist/t_hist (device,
 * nsteps doubles each, may be NULL) receive the accepted dt and the time after
 * each step.  h_force (device, nsteps doubles, normally NULL) replays a
 * prescribed step sequence: step s takes h_force[s] in one attempt, whatever
 * its error (used to compare arithmetic precisions on identical steps; the
 * reference has no such mode).  Per accepted step two launches are queued:
 * the traction product, then one cooperative kernel with the retry loop of
 * Dormand-Prince attempts (max-relative error norm) and the state update
 * (src/QDsim_gpu.py:942-1027, 1128-1262); dt, time and the attempt count
 * carry over in ctrl.  Asynchronous on `stream`: the return value reports the
 * launches; the outcome of the steps is ctrl->status (read it after the
 * stream; after a failed step the remaining launches return at once). */
int pq3d_dense_step(const pq3d_dense_sim *sim, int nsteps, double *h_hist, double *t_hist,
                    const double *h_force, void *stream);

/* ---------------- device: batched ensemble (B runs, one mesh) ---------------- */

/* Per-run control block (device memory, one per run). */
typedef struct pq3d_run_ctrl {
    double h;              /* trial dt of the next attempt (dttry, then dtnext) */
    double time;           /* simulated time (s) */
    double t_end;          /* the run retires once time >= t_end */
    double h_last;         /* dt of the last accepted step */
    int64_t attempts;      /* attempted steps (7 right-hand-side evaluations each) */
    int64_t steps;         /* accepted steps */
    int64_t max_steps;     /* the run retires after this many accepted steps */
    uint64_t err1_bits;    /* max-error reduction of the current attempt (double bits) */
    uint64_t err2_bits;
    int32_t status;        /* PQ3D_OK or PQ3D_ERR_STEP */
    int32_t active;        /* 1 while the run steps */
    int32_t nrjct;         /* rejected attempts of the current step */
    int32_t accepted;      /* 1 if the last attempt was accepted */
} pq3d_run_ctrl;

/* Traction-product operand precision of the batched stepper. */
#define PQ3D_BATCH_FP64 0      /* FP64 operator, FP64 FMA (CUDA cores) */
#define PQ3D_BATCH_FP32 1      /* FP32 operator, FP32 FMA (CUDA cores), FP64 across chunks */
#define PQ3D_BATCH_BF16X6 2    /* FP32 operator split on the fly into 3 BF16 pieces, v' into 3 BF16
                                  pieces, the 6 leading cross products on tcgen05 tensor cores,
                                  FP32 accumulation in tensor memory, K slices added in
                                  float-float */
#define PQ3D_BATCH_HMAT 3      /* H-matrix product (pq3d_hmat_apply); K points to a host pq3d_hmat */
#define PQ3D_BATCH_BF16X18 4   /* operator (32 bits per row and 1024-column chunk) and v' (48 bits per
                                  run and 256-column span) as exact fixed-point BF16 slices; the 18
                                  slice products down to 2^-40 of the leading one on tcgen05 tensor
                                  cores, exact accumulation per span, spans added in float-float:
                                  the FP64 product to ~2^-32 of each chunk's largest operator entry
                                  (static) and ~2^-40 of each span's largest v' (dynamic).  B <= 64,
                                  no row shards */

/* Device state of B simulations sharing one mesh.  Arrays are run-major
 * [B][N] FP64 unless stated.  Same fields and units as pq3d_dense_sim. */
typedef struct pq3d_batch_sim {
    int64_t N;
    int32_t B;
    int32_t precision;     /* PQ3D_BATCH_* */
    double *Tno, *Tt1o, *Tt2o, *state, *slipv1, *slipv2, *slipv, *slip1, *slip2;
    const double *a, *b, *dc, *f0, *shear_loading, *normal_loading, *cos_rake0, *sin_rake0;
    double *rates;         /* partial traction rates, room for nsplit x Bp x 3N doubles: FP64 [Bp][3N]
                              (nsplit = 1) for FP64 and HMAT; FP64 [nsplit][Bp][3N] for FP32 (the K
                              slices' sums, added in slice order by the stepper); for BF16X6 FP32
                              [nsplit][Bp][3N], the K slices' tensor-memory sums, added in
                              float-float by the stepper; for BF16X18 float2 (hi, lo)
                              [nsplit][Bp][3N], float-float K-slice sums */
    int32_t nsplit;        /* K-slices of the operator product: >= 1 for BF16X6 and BF16X18, 1..64 for
                              FP32, 1 for FP64 and HMAT */
    int32_t tc_ctas;       /* BF16X6: CTAs per SM of the tensor-core product, 0 (= 2) or 1..3; the launch
                              shape only, results do not depend on it */
    double *cand;          /* [B][N][4] candidate state */
    void *vop;             /* operator-product right-hand side of all runs, padded to Bp = B rounded up
                              to 16 runs (extra runs zero): FP64 [Bp][2N], FP32 [Bp][2N], for
                              BF16X6 the packed pieces (pq3d_batch_rhs_bytes, zero-initialised),
                              for BF16X18 the packed fixed-point slices (pq3d_batch_rhs_fix_bytes) */
    const void *K;         /* operator: FP64 (3N)x(2N) for FP64, FP32 (3N)x(2N) for FP32, the
                              packed BF16 pieces (pq3d_batch_pack_operator) for BF16X6, the packed
                              fixed-point slices (pq3d_batch_pack_operator_fix) for BF16X18, a host
                              pointer to a pq3d_hmat for HMAT (v' then FP64 [Bp][2N]) */
    pq3d_run_ctrl *ctrl;   /* [B] */
    double V0, Vpl, eta;
    int32_t fix_Tn;
    int32_t attempt64;     /* FP32, BF16X6, BF16X18, HMAT: 1 = Dormand-Prince stages in the reference
                              FP64 arithmetic, 2 = in float-float on the FP32 pipes (the FP64
                              attempt's accuracy: exponent arguments reduced in FP64 once per
                              attempt), base unused (may be NULL) for both; 0 = mixed precision */
    /* Receiver-row shard (FP64 and FP32 only): this process steps cells
     * [cell0, cell0 + N) of an N_total-cell mesh.  The per-cell arrays, cand
     * and rates hold the shard's N cells; K holds the shard's 3N rows of the
     * (3 N_total) x (2 N_total) operator; vop holds v' of ALL N_total cells
     * ([Bp][2 N_total]), of which the shard writes its own slice and the
     * caller exchanges the rest (allgather) after each iteration.  N_total = 0
     * means an unsharded simulation (N_total = N, cell0 = 0). */
    int64_t N_total;
    int64_t cell0;
    /* Mixed precisions (FP32, BF16X6, HMAT with attempt64 = 0): the cells'
     * start-of-step constants of the mixed-precision Dormand-Prince attempt,
     * FP32 [PQ3D_BATCH_BASE_FIELDS][B][N], written by pq3d_batch_prepare and
     * by the update of every accepted step.  NULL (unused) otherwise. */
    float *base;
    /* BF16X18: the cell order of the fixed-point product (device int64, NULL =
     * identity): fix_order[p] = cell at position p of the packed operator's
     * rows and columns, fix_pos[cell] = its position.  A spatially compact
     * order (pq3d_hmat_cluster_order) keeps each 256-column span, whose
     * largest |v'| sets the span's fixed-point grid, and each 1024-column
     * operator chunk inside one region of the fault; the mesh order of a long
     * fault puts far-apart cells in one span, and the slow cells sharing a
     * span with a nucleating patch keep only the bits of their v' below the
     * patch's. */
    const int64_t *fix_order;
    const int64_t *fix_pos;
} pq3d_batch_sim;

#define PQ3D_BATCH_BASE_FIELDS 24

/* Packed operator of the tensor-core product: the FP64 operator split into
 * three BF16 pieces, stored as [3N/128 tiles][2N/32 blocks][3][128 x 32]
 * shared-memory images (8-row x 16-byte core matrices).  Bytes, and the packing
 * kernel (run once after assembly). */
size_t pq3d_batch_operator_bytes(int64_t N);
int pq3d_batch_pack_operator(const double *K64, int64_t N, void *Kpacked, void *stream);
/* Bytes of the packed right-hand side for B runs (BF16X6). */
size_t pq3d_batch_rhs_bytes(int64_t N, int B);
/* The tensor-core product alone: FP32 out[(s*Bp + n)*3N + m] (s < nsplit K
 * slices, Bp = B rounded up to 16) from the packed operator and right-hand
 * side.  nsplit sets the order in which the slices' sums are added (and so
 * the bits of the result); ctas_per_sm (0 = 2, else 1..3) is the launch shape
 * only. */
int pq3d_batch_gemm_bf16x6(const void *Kpacked, const void *Vpacked, int64_t N, int B, int nsplit, int ctas_per_sm,
                           float *out, void *workspace, size_t workspace_bytes, void *stream);
/* The launch of that product for B runs on the current device: plan[0] = CTAs
 * per SM actually launched for the requested ctas_per_sm (fewer where shared
 * or tensor memory does not fit them), plan[1] = pipeline stages per CTA. */
int pq3d_batch_gemm_bf16x6_plan(int B, int ctas_per_sm, int32_t *plan);

/* Packed operator of the fixed-point tensor-core product (BF16X18): per operator
 * row and 1024-column chunk one exponent e (|K| < 2^e over the chunk) and four
 * BF16 slices d_p 2^(e-7-8p), |d_p| <= 128, stored as [3N/128 tiles][2N/32
 * blocks][4][128 x 32] shared-memory images.  Bytes, and the packing kernel
 * (once per mesh; the operator rounded to 32 bits of its chunk's largest entry). */
size_t pq3d_batch_operator_fix_bytes(int64_t N);
/* order (device int64 [N], NULL = identity): order[p] = cell at position p;
 * the packed operator holds rows 3 order[p] + c and columns 2 order[q] + s at
 * positions 3p + c and 2q + s, and the product's outputs come in that row
 * order. */
int pq3d_batch_pack_operator_fix(const double *K64, int64_t N, const int64_t *order, void *Kpacked, void *stream);
/* Bytes of the packed fixed-point right-hand side for B <= 64 runs (padded to
 * 32 or 64 runs), and its packing from v ([B][2N] FP64 device array,
 * v[r][2j + s]): per run and 256-column span six slices (48 bits of the span's
 * largest |v|).  The batched stepper packs v' itself; this entry serves the
 * product alone. */
size_t pq3d_batch_rhs_fix_bytes(int64_t N, int B);
int pq3d_batch_pack_rhs_fix(const double *v, int64_t N, int B, const int64_t *order, void *Vpacked, void *stream);
/* The fixed-point tensor-core product alone: out[((s*Bp + n)*3N + m)*2 + {0,1}]
 * = (hi, lo) FP32, s < nsplit, Bp = B rounded up to 16, B <= 64; the nsplit
 * partial sums add up to sum_k K[m][k] v[n][k], the exact product of the
 * slices up to ~2^-44 relative.  A partial sum is either K slice s (column
 * blocks 2N/32 s / nsplit .. 2N/32 (s+1) / nsplit, one CTA per 128-row tile and
 * slice) or, when no 128-row tile meets more than nsplit shares of the
 * balanced grid (one CTA per SM, each streaming an equal share of the
 * tile-major 32-column blocks), the s-th share of the row's tile, zero past
 * its last share.  Six wide tcgen05.mma per 16-column step (one per operator
 * slice and run of right-hand-side slices, accumulating in tensor-memory slots
 * by level); nsplit sets the schedule and the order of the partial sums. */
int pq3d_batch_gemm_bf16x18(const void *Kpacked, const void *Vpacked, int64_t N, int B, int nsplit, float *out,
                            void *workspace, size_t workspace_bytes, void *stream);
/* Device workspace bytes of one batched iteration (GEMM split-K partials live in
 * sim->rates; this is what the tensor-core product needs besides). */
size_t pq3d_batch_workspace_bytes(const pq3d_batch_sim *sim);

/* Prepare the operator right-hand side from the current slip rates and, for
 * the mixed precisions, the start-of-step constants from the current state
 * (run once before the first iteration and after any host-side change of
 * the state). */
int pq3d_batch_prepare(const pq3d_batch_sim *sim, void *stream);

/* One batched iteration on `stream`, graph-capturable: the operator product
 * for all runs, one Dormand-Prince attempt per active run with its own dt,
 * the per-run accept/reject decision and the state update of the accepted runs
 * (masked acceptance; rejected runs retry with their smaller dt next time). */
int pq3d_batch_iterate(const pq3d_batch_sim *sim, void *workspace, size_t workspace_bytes, void *stream);

/* The same iteration in two halves, for row-sharded simulations: _begin does
 * the operator product and the attempt and leaves each run's max error norms
 * of this shard in ctrl[r].err1_bits / err2_bits (FP64 bit patterns, order-
 * preserving as signed 64-bit integers); the caller reduces them with MAX over
 * the shards and writes the result back; _end decides and updates.  The
 * decision only reads the control record, so every shard takes the same one.
 * pq3d_batch_iterate = _begin + _end. */
int pq3d_batch_iterate_begin(const pq3d_batch_sim *sim, void *workspace, size_t workspace_bytes, void *stream);
int pq3d_batch_iterate_end(const pq3d_batch_sim *sim, void *stream);

/* ---------------- device: H-matrix ---------------- */

/* Source and receiver tables of a mesh (the set-up step of the assembly) into
 * `workspace` (pq3d_gf_workspace_bytes(N)), and with halfspace != 0 the image
 * and free-surface tables: used by the H-matrix kernels. */
int pq3d_gf_setup(const double *nodes, const int64_t *tris, int64_t N, int halfspace, void *workspace,
                  size_t workspace_bytes, void *stream);

/* H-matrix of the (3N)x(2N) traction operator in a renumbering where every
 * cluster is a contiguous range (perm[p] = element at position p).  Replaces
 * the reference's BlockTree (src/Hmatrix.py:277-2196) for the product. */
typedef struct pq3d_hmat {
    int64_t N;
    int32_t nblocks, nleaves;
    int64_t t_rows;               /* sum of the ranks of the low-rank blocks */
    const int64_t *perm;          /* [N] */
    const int64_t *blk;           /* [nblocks][4]: r0, r1, c0, c1 (permuted element ranges) */
    const int32_t *rank;          /* [nblocks]: rank k >= 0 of a low-rank block, -1 for a dense block */
    const int64_t *off;           /* [nblocks]: offset (floats) of the block in data */
    const float *data;            /* FP32: dense block (3m x 2n, column-major) or U (3m x k, column-major)
                                     then V (k x 2n, row-major) */
    const int32_t *lr_ids;        /* low-rank block ids, in order */
    const int64_t *t_info;        /* [t_rows][2] per rank row (low-rank blocks in lr_ids order): offset of its V
                                     row in data, then (first column 2 c0) | (row length 2n) << 32 */
    const int64_t *t_off;         /* [nblocks]: first rank row of the block in the product workspace */
    const int64_t *leaf;          /* [nleaves][2]: permuted ranges of the leaf row clusters */
    const int64_t *leaf_ptr;      /* [nleaves + 1] */
    const int32_t *leaf_blocks;   /* blocks whose row range covers each leaf row cluster, fixed order */
    const int32_t *t_sched;       /* [t_rows] rank rows: those of at most 8192 columns, then the longer ones */
    int64_t t_nlong;              /* number of the longer rows (the tail of t_sched) */
    const int64_t *t_grp;         /* [t_ngrp][2] groups of up to 4 consecutive shorter rank rows of one block
                                     (they share their x values), 16-byte aligned: V offset of the first row
                                     (< 2^40) | row length << 40 | group size << 56, then first column
                                     2 c0 | first rank row << 32 */
    int64_t t_ngrp;
} pq3d_hmat;

/* Cluster and block tree of the H-matrix on the device (replaces the host
 * recursions createHmatrix / build_block_tree / create_recursive_blocks,
 * src/Hmatrix.py:143-192, 2077-2196, with their rules: bisection of the
 * longest bounding-box axis at its midpoint, min_size points per leaf
 * cluster, admissibility min(diam) <= eta * dist, mini_leaf).  xg: [N][3]
 * centroids (device, FP64).  Outputs (device): perm[N] (element at each
 * position of the depth-first leaf order), leaves [N][2] capacity (leaf
 * cluster ranges, *n_leaves of them), blocks [cap_blocks][5] (r0, r1, c0, c1,
 * lowrank; depth-first order, *n_blocks of them).  With a blocks array too
 * small, returns PQ3D_ERR_ARG with *n_blocks set to the size needed.
 * *depth (may be NULL) = cluster-tree levels.  Allocates its scratch; reads
 * one count per level back to the host (synchronises `stream`). */
/* The cluster tree alone: perm[N] (device) = the depth-first leaf order of
 * the bisection tree with leaves of <= min_size points -- a spatially compact
 * order of the elements (the BF16X18 product's fix_order). */
int pq3d_hmat_cluster_order(const double *xg, int64_t N, int min_size, int64_t *perm, int32_t *depth, void *stream);
int pq3d_hmat_partition(const double *xg, int64_t N, int min_size, int mini_leaf, double eta, int64_t *perm,
                        int64_t *leaves, int64_t *n_leaves, int64_t *blocks, int64_t cap_blocks, int64_t *n_blocks,
                        int32_t *depth, void *stream);
/* ACA (partial pivoting, relative Frobenius tolerance `tol`) of the listed
 * admissible blocks, one CTA per block, rows and columns generated by the GF
 * kernel from `tables` (pq3d_gf_setup).  Per block b: kcap[b] = rank cap,
 * UV + uv_off[b] = FP64 scratch for U (kcap x 3m) then V (kcap x 2n),
 * used + used_off[b] = 3m zeroed bytes.  Outputs rank[b] and status[b]
 * (0 converged, 1 rank cap reached, 2 non-finite).  Replaces ACA_worker /
 * ACA_plus_full_traceS/D (src/Hmatrix.py:661-1344). */
int pq3d_hmat_aca(const double *tables, int64_t N, const int64_t *perm, int nblocks, const int64_t *blk,
                  const int32_t *kcap, double tol, double mu, double lambda_, int halfspace, double *UV,
                  const int64_t *uv_off, uint8_t *used, const int64_t *used_off, int32_t *rank, int32_t *status,
                  void *stream);
/* Dense blocks ids[0..nids) into D + d_off[b] (FP32, column-major: element
 * (row, col) at col * 3m + row). */
int pq3d_hmat_dense_blocks(const double *tables, int64_t N, const int64_t *perm, const int64_t *blk,
                           const int32_t *ids, int nids, double mu, double lambda_, int halfspace, float *D,
                           const int64_t *d_off, void *stream);
/* FP64 ACA factors of blocks ids[] -> FP32 U (column-major, 3m x k) and V (k x 2n) at out + out_off[b]. */
int pq3d_hmat_pack_factors(const double *UV, const int64_t *uv_off, const int64_t *blk, const int32_t *kcap,
                           const int32_t *rank, const int32_t *ids, int nids, float *out, const int64_t *out_off,
                           void *stream);
/* Y[r] = H X[r] for B right-hand sides: X [B][2N] (element order, interleaved
 * strike/dip), Y [B][3N] (traction components per element).  Deterministic:
 * each output row adds its blocks in a fixed order with compensated FP32
 * arithmetic.  Replaces blocks_process_MVM (src/Hmatrix.py:1773-1866), all six
 * operator types at once. */
size_t pq3d_hmat_workspace_bytes(const pq3d_hmat *H, int B);
/* The same for the runs r with run_active[r * active_stride] != 0 only (device
 * int32 flags, e.g. the `active` field of a pq3d_run_ctrl array; the rows of
 * the other runs are left untouched). */
int pq3d_hmat_apply_masked(const pq3d_hmat *H, const double *X, int B, double *Y, const int32_t *run_active,
                           int active_stride, void *workspace, size_t workspace_bytes, void *stream);
int pq3d_hmat_apply(const pq3d_hmat *H, const double *X, int B, double *Y, void *workspace, size_t workspace_bytes,
                    void *stream);

/* ---------------- self-tests of the bounded device waits ---------------- */
/* No counterpart in the reference (it has no device waits).  A cooperative
 * launch of `nblocks` blocks (<= 64) in which every block but `skip_block`
 * arrives at one grid barrier -- the barrier of the dense stepper -- with the
 * wait limit lowered to `spin_limit` iterations (~1 us each; <= 65536):
 * returns PQ3D_ERR_TIMEOUT (the status the stepper records) once the waits
 * give up; returned_host[b] (host, nblocks ints) = 1 if block b returned
 * after giving up, 2 if it passed the barrier, 3 for the block that skipped
 * it.  Allocates a small buffer. */
int pq3d_selftest_barrier_timeout(int nblocks, int skip_block, unsigned spin_limit, int *returned_host);
/* One block of 128 threads waits, with the bounded mbarrier wait of the
 * tensor-core products and its limit lowered to `wait_limit` tries (<= 65536),
 * on an mbarrier nobody arrives at: returns PQ3D_ERR_TIMEOUT with the error
 * word set, *gave_up_host = the threads that gave up (128). */
int pq3d_selftest_mbar_timeout(unsigned wait_limit, int *gave_up_host);
/* The FP64 <-> float-float conversions of the float-float attempt (integer
 * bit operations on the device) on n host values (n <= 2^20): ff_host[2i],
 * ff_host[2i+1] = (hi, lo) of x_host[i]; d_host[i] = f_host[i] widened to
 * FP64; h_host[i] = |(x_host[i], y_host[i])| by the float-float norm of the
 * update kernel.  Allocates small buffers. */
int pq3d_selftest_ff_conversions(const double *x_host, const float *f_host, const double *y_host, int n,
                                 float *ff_host, double *d_host, double *h_host);
/* The configuration test of the dense assembly (coordinates from the
 * reciprocal of the barycentric denominator, decisions in FP32 where the
 * coordinates are well separated, else the division-based test) and the
 * division-based test of src/TDstressFS_C.cpp:125-166 on n host points
 * (n <= 2^22), pts_host[8i..8i+7] = (x, y, z, p1y, p1z, p3y, p3z, den):
 * fast_host[i], exact_host[i] in {1, -1, 0}.  Allocates small buffers. */
int pq3d_selftest_tri_mode(const double *pts_host, int n, int *fast_host, int *exact_host);

#ifdef __cplusplus
}
#endif
#endif /* PQ3D_H */
