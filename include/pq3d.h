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
#define PQ3D_ERR_UNSUPPORTED 5  /* a feature this build does not provide */

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

/* Host-buffer variant for callers that keep the mesh and the operator in host
 * memory (the reference keeps A1s..Bd as NumPy arrays): copies the mesh in,
 * assembles in row blocks on two streams and copies each block back while the
 * next one is computed.  K64_host: (3N)x(2N) doubles (pinned memory recommended);
 * K32_host may be NULL.  Allocates and frees its own device buffers. */
int pq3d_assemble_dense_host(const double *nodes_host, int64_t n_nodes, const int64_t *tris_host,
                             int64_t N, double mu, double lambda_, int halfspace,
                             double *K64_host, float *K32_host);

/* ---------------- device: dense stepping (plain FP64) ---------------- */

/* out[r] = sum_c K[r][c] * v[c] for the (3N) x (2N) FP64 operator: the traction
 * product K.(V - Vpl) of src/QDsim_gpu.py:948-957 (v interleaved [j][strike,dip]). */
int pq3d_dense_matvec_f64(const double *K64, int64_t N, const double *v, double *out, void *stream);
/* Same with the FP32 operator copy: compensated FP32 products and sums (the
 * FP32-rounded operator applied to v to ~2^-44 relative). */
int pq3d_dense_matvec_f32(const float *K32, int64_t N, const double *v, double *out, void *stream);

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
    /* scratch: vprime[2N], cand[4N] */
    double *vprime, *cand;
    /* FP64 operator (3N)x(2N) or FP32 operator (exactly one non-NULL) */
    const double *K64;
    const float *K32;
    /* device control block: see pq3d_step_ctrl */
    struct pq3d_step_ctrl *ctrl;
    /* scalars */
    double V0, Vpl, eta;   /* eta = mu / (2 cs) */
    int fix_Tn;
} pq3d_dense_sim;

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
 * reference has no such mode).  One cooperative persistent kernel does, per accepted step, the
 * traction product, the retry loop of Dormand-Prince attempts with the
 * max-relative error norm, and the state update (src/QDsim_gpu.py:942-1027,
 * 1128-1262).  Asynchronous on `stream`: the return value reports the launch;
 * the outcome of the steps is ctrl->status (read it after the stream). */
int pq3d_dense_step(const pq3d_dense_sim *sim, int nsteps, double *h_hist, double *t_hist,
                    const double *h_force, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PQ3D_H */
