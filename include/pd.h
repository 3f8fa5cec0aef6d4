/*
 * pd.h — C ABI of the GB300 peridynamics engine (libpd_gb300.so).
 *
 * The reference (XiaoMmingW/PD_Gpu1) exposes no plugin layer: its operator API
 * is a set of free host launchers over raw SoA device pointers plus a global
 * `__constant__ device_parameter dp` (Base.cuh:46-70).  This header replaces
 * those launchers one for one with status-returning entry points over an
 * opaque context that owns the device memory.  Every entry point cites the
 * reference interface it replaces.
 *
 * Conventions
 *   - All floating point is FP64 (the reference built with -DDOUBLE_PRECISION).
 *   - Node fields are indexed in the reference's node order; bond fields are in
 *     CSR order: row i holds the bond family of node i sorted by ascending
 *     neighbour id, which is exactly the row order of the reference's CPU
 *     neighbour list (Neighbor.cu:42-80).
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *   - Every call returns PD_OK (0) or a negative PD_ERR_* code; nothing exits
 *     the process (the reference's CHECK macro calls exit(1), Error.cuh:9-23).
 *   - One context per host thread at a time; contexts are independent.
 */
#ifndef PD_GB300_H
#define PD_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define PD_OK 0
#define PD_ERR_ARG -1           /* bad argument (null pointer, bad size, bad enum)   */
#define PD_ERR_CUDA -2          /* a CUDA runtime call failed (see pd_last_error)    */
#define PD_ERR_STATE -3         /* call out of order (e.g. force before neighbours)  */
#define PD_ERR_FAMILY -4        /* a node has more than MN neighbours (ELL overflow)  */
#define PD_ERR_NONFINITE -5     /* NaN/Inf found by pd_check_finite                   */
#define PD_ERR_NOMEM -6         /* device allocation failed                           */
#define PD_ERR_TIMEOUT -7       /* a bounded device-side wait gave up                 */
#define PD_ERR_UNSUPPORTED -8   /* combination not implemented (e.g. 1-D models)      */

/* ---- enums ------------------------------------------------------------- */
/* Dselect::B_S (Base.cuh:35-43) */
#define PD_MODEL_BOND 1   /* bond-based prototype micro-elastic brittle (PMB) */
#define PD_MODEL_STATE 2  /* ordinary state-based (LPS)                       */
/* Dselect::Mode */
#define PD_MODE_STATIC 1  /* quasi-static, adaptive dynamic relaxation (ADR) */
#define PD_MODE_DYNAMIC 2 /* explicit velocity-Verlet                         */

/* Field identifiers for pd_get_field / pd_set_field / pd_field_ptr.
 * Node fields hold N doubles per component (x, y[, z] stored as separate
 * arrays, like BAtom, Base.cuh:186-225); bond fields hold B entries. */
typedef enum pd_field {
    PD_F_X = 0, PD_F_Y, PD_F_Z,                  /* reference coordinates          */
    PD_F_UX, PD_F_UY, PD_F_UZ,                   /* displacement disp_*            */
    PD_F_VX, PD_F_VY, PD_F_VZ,                   /* velocity vel_*                 */
    PD_F_AX, PD_F_AY, PD_F_AZ,                   /* acceleration acc_*             */
    PD_F_FX, PD_F_FY, PD_F_FZ,                   /* peridynamic force pforce_*     */
    PD_F_BX, PD_F_BY, PD_F_BZ,                   /* body force bforce_*            */
    PD_F_VHX, PD_F_VHY, PD_F_VHZ,                /* ADR velhalfold_*               */
    PD_F_FOX, PD_F_FOY, PD_F_FOZ,                /* ADR pforceold_*                */
    PD_F_DMG,                                    /* damage dmg                     */
    PD_F_M, PD_F_THETA,                          /* state-based m, theta           */
    PD_F_FNCST_X, PD_F_FNCST_Y, PD_F_FNCST_Z,    /* surface-correction factors     */
    /* integer node field */
    PD_F_NN,                                     /* family size NN (int32)         */
    /* bond fields (CSR order) */
    PD_F_ROWPTR,                                 /* int64[N+1]                     */
    PD_F_NL,                                     /* neighbour id, int32[B]         */
    PD_F_IDIST,                                  /* |xi|, double[B]                */
    PD_F_FAC,                                    /* volume correction, double[B]   */
    PD_F_SCR,                                    /* surface correction, double[B]  */
    PD_F_W,                                      /* influence w, double[B]         */
    PD_F_E,                                      /* extension e, double[B]         */
    PD_F_FAIL,                                   /* 1 intact / 0 broken, int32[B]  */
    PD_F_COUNT
} pd_field;

/* ---- parameters -------------------------------------------------------- */
/* The first block mirrors device_parameter (Base.cuh:46-68) field for field;
 * the rest carries what the reference keeps in Dselect, BaseModel_Parameter
 * or hard-codes in its kernels. */
typedef struct pd_params {
    double pi;
    int32_t N, MN, N_int, nx, ny, nz;
    double dx, emod, dens, pratio, bc, delta, critical_s, vol, dt;
    int32_t nt;
    int32_t dim;          /* Dselect::Dim: 2 or 3 */
    double mass, K, G;
    /* extensions */
    int32_t model;        /* PD_MODEL_*  (Dselect::B_S)  */
    int32_t mode;         /* PD_MODE_*   (Dselect::Mode) */
    double thick, length, height, width, load;
    double sedload;       /* surface-correction test energy: 2-D 0.5E/(1-v^2)1e-6 (Surf_Corr.cu:238), 3-D 0.6E1e-6 (:280) */
    double break_ymin;    /* 3-D bonds break only when both ends have y >= break_ymin
                             (Force_Bond.cu:117, Force_State.cu:280 hard-code -0.04); -1e300 disables */
} pd_params;

/* BaseModel_Parameter::cal_parameter (Base.cuh:114-183) + initialil_parameter
 * (Base_Function.cu:14-36): derive N, MN, nx, ny, nz, delta, bc, vol, mass, K, G
 * from the driver inputs.  fix_k3d=0 keeps the reference's 3-D state-based bulk
 * modulus K = E/3/(1-2G) (Base.cuh:175); fix_k3d=1 uses K = E/(3(1-2v)). */
int pd_params_derive(pd_params* p, int dim, int model, int mode, double dt, double nt, double dx,
                     double load, double thick, double length, double height, double width,
                     double emod, double pratio, double dens, double critical_s, int fix_k3d);

/* ---- context ----------------------------------------------------------- */
typedef struct pd_ctx pd_ctx;

/* Base_Allocate (Memory.cu:139-147): allocates every node field for p->N nodes.
 * Bond storage is allocated by pd_find_neighbor once the family size is known. */
pd_ctx* pd_create(const pd_params* p, int* status);
/* Base_Free (Memory.cu:276-284, which re-allocates instead of freeing). */
int pd_destroy(pd_ctx* ctx);
/* Test hook (no reference counterpart): from now on, the n-th device
 * allocation of pd_create (counting from 0) is refused once, as if the device
 * were out of memory, and that pd_create returns NULL with PD_ERR_NOMEM after
 * releasing what it had allocated; n = -1 clears the hook.  Lets a caller
 * check the clean-up of a partly built context without exhausting a GPU. */
int pd_debug_fail_allocation(int n);
int pd_get_params(const pd_ctx* ctx, pd_params* out);
/* Replace the parameters (same N/dim/model; a batch keeps its dt);
 * cudaMemcpyToSymbol(dp, ...) of the drivers. */
int pd_set_params(pd_ctx* ctx, const pd_params* p);
const char* pd_last_error(const pd_ctx* ctx);
const char* pd_status_string(int status);

/* Copy a field between host memory and the context (count elements, checked
 * against the field's size).  Replaces the cudaMemcpy calls of Save.cu and
 * of the drivers' setup (Solve_Kalthoff_Winkler.cu:381-383). */
int pd_get_field(pd_ctx* ctx, int field, void* host, size_t count, void* stream);
int pd_set_field(pd_ctx* ctx, int field, const void* host, size_t count, void* stream);
/* Device pointer and element count of a field (for zero-copy interop). */
int pd_field_ptr(pd_ctx* ctx, int field, void** dev, size_t* count);
/* Number of directed bonds B (0 before pd_find_neighbor). */
int64_t pd_num_bonds(const pd_ctx* ctx);
/* Wait for all work on the stream. */
int pd_sync(pd_ctx* ctx, void* stream);

/* ---- geometry (Coord.cu) ----------------------------------------------- */
/* kernel_Initial_coord_plate / Initial_coord_plate_cpu (Coord.cu:6-28). */
int pd_coord_plate(pd_ctx* ctx, void* stream);
/* kernel_coord_plate_crack / coord_plate_crack_cpu (Coord.cu:34-66):
 * interior rows, then 3 rows above and 3 rows below stored after N_int. */
int pd_coord_plate_crack(pd_ctx* ctx, void* stream);
/* coord_KW (Coord.cu:77-129): host-side generator for the notched slab.  Writes
 * up to `cap` nodes into x,y,z (host arrays) and returns the node count in *n. */
int pd_coord_kw(const pd_params* p, double rad, double* x, double* y, double* z, int64_t cap, int64_t* n);

/* ---- neighbour family (Neighbor.cu) ------------------------------------ */
/* find_neighbor_gpu (Neighbor.cu:82-90), kernel_find_neighbor_2D/3D (:7-40):
 * cell-list build of the bond family |xj-xi|^2 < delta^2 into CSR, each row
 * sorted ascending.  Also allocates all bond arrays and sets every fail flag
 * to 1 (kernel_initial_fail, Initial.cu:6-14).  Returns PD_ERR_FAMILY if a
 * row exceeds p->MN (the reference's ELL would overflow, Neighbor.cu:18). */
int pd_find_neighbor(pd_ctx* ctx, void* stream);

/* ---- setup passes ------------------------------------------------------ */
/* kernel_vol_Corr (Surf_Corr.cu:7-35): idist and fac per bond. */
int pd_vol_corr(pd_ctx* ctx, void* stream);
/* surface_correct_gpu (Surf_Corr.cu:235-310): vol_Corr + per-axis strain
 * energy factors fncst + per-bond scr, fused into two kernels (one family
 * pass, then the coefficient pass, which needs both end nodes' fncst).  In a
 * state-based context the family pass also writes w and m. */
int pd_surface_correct(pd_ctx* ctx, void* stream);
/* kernel_initial_weight_2D/3D (Force_State.cu:8-54): w per bond, m per node,
 * in one family pass with vol_Corr's idist and fac (a preceding
 * pd_vol_corr is not needed; after one the values are rewritten unchanged). */
int pd_initial_weight(pd_ctx* ctx, void* stream);
/* kernel_set_crack_2D (Base_Function.cu:39-81): cut bonds crossing a segment
 * of length clength centred at (loc_x, loc_y) at angle theta (radians). */
int pd_set_crack_2d(pd_ctx* ctx, double clength, double loc_x, double loc_y, double theta, void* stream);
/* kernel_set_crack (Solve_Kalthoff_Winkler.cu:40-63): notch cut at x = +-rad. */
int pd_set_crack_kw(pd_ctx* ctx, double rad, void* stream);
/* base_integrate_initial_gpu / static_initial_bond_gpu (Initial.cu:24-75):
 * zero disp, vel, acc, bforce, pforce (+ ADR state). */
int pd_initial_state(pd_ctx* ctx, void* stream);
/* Build the per-bond coefficients the force kernels read (from idist, fac,
 * scr, w, m).  Called implicitly by the first force call after setup changes. */
int pd_prepare(pd_ctx* ctx, void* stream);

/* ---- forces ------------------------------------------------------------ */
/* bond_force_2D_gpu / bond_force_3D_gpu (Force_Bond.cu:143-157);
 * kernel_particle_force_2D (:52-85), kernel_bond_force_3D (:87-141):
 * PMB force density on nodes [0, N_int) and breakage s > critical_s. */
int pd_bond_force(pd_ctx* ctx, void* stream);
/* kernel_cal_theta_2D/3D + kernel_state_force_2D/3D (Force_State.cu:56-134,
 * :203-306): dilatation on all N nodes, force and breakage on [0, N_int). */
int pd_state_force(pd_ctx* ctx, void* stream);

/* ---- integration and reductions (Integrate.cu, Reduce.cu) -------------- */
/* static_integrate_gpu (Integrate.cu:130-172): kernel_cnn + cal_cn + kernel_integrate.
 * The damping coefficient stays on the device (no host sync). ct is the step index. */
int pd_integrate_adr(pd_ctx* ctx, int ct, void* stream);
/* Last damping coefficient cn (Integrate.cu:108-129), copied to the host (syncs). */
int pd_get_adr_cn(pd_ctx* ctx, double* cn, void* stream);
/* kernel_integrate_2D_1 / 3D_1 (Integrate.cu:174-216): v += dt/2 a; u += v dt. */
int pd_integrate_verlet1(pd_ctx* ctx, void* stream);
/* kernel_integrate_2D_2 / 3D_2 (Integrate.cu:218-266): a = (F+b)/rho; v += dt/2 a. */
int pd_integrate_verlet2(pd_ctx* ctx, void* stream);
/* sum (Reduce.cu:52-65): sum of n doubles of a device array into *result
 * (host).  Deterministic order. */
int pd_reduce_sum(pd_ctx* ctx, const double* dev_x, int64_t n, double* result, void* stream);

/* ---- damage, loads, contact ------------------------------------------- */
/* kernel_cal_dmg_2D/3D (Base_Function.cu:149-217). */
int pd_damage(pd_ctx* ctx, void* stream);
/* kernel_quick_load (Solve_Plate_Crack_Grow.cu:8-19): boundary rows after
 * N_int move by +-load*dt in y. */
int pd_quick_load(pd_ctx* ctx, double load, void* stream);
/* load_plate_tensile_gpu (Solve_Plate_Tensile.cu:7-17): bforce_x = -+0.001E/dx
 * on the left and right columns. */
int pd_load_plate_tensile(pd_ctx* ctx, void* stream);

/* Rigid cylindrical impactor of the Kalthoff-Winkler driver
 * (Cylinder_Parameter, Base.cuh:227-246). */
typedef struct pd_cylinder {
    double rad, mass, height, v, x, y, z;
    double vel[3], disp[3], acc[3], force[3];
} pd_cylinder;
/* kernel_initial_cylinder (Solve_Kalthoff_Winkler.cu:9-22). */
int pd_cylinder_init(pd_ctx* ctx, const pd_cylinder* cyl, void* stream);
int pd_cylinder_get(pd_ctx* ctx, pd_cylinder* cyl, void* stream);
/* kernel_cy_integrate_1 (Solve_Kalthoff_Winkler.cu:89-99). */
int pd_cylinder_integrate1(pd_ctx* ctx, void* stream);
/* kernel_contact (Solve_Kalthoff_Winkler.cu:112-175): project penetrating
 * nodes onto the cylinder, reaction force summed on the device. */
int pd_contact(pd_ctx* ctx, void* stream);
/* kernel_cy_integrate_2 (Solve_Kalthoff_Winkler.cu:242-253). */
int pd_cylinder_integrate2(pd_ctx* ctx, void* stream);

/* ---- fused time stepping ---------------------------------------------- */
/* Per-step body of solve_plate_tensile's loop (Solve_Plate_Tensile.cu:106-131)
 * for nsteps ADR steps starting at step index ct0: force + damping + update,
 * two kernels per step, optionally with boundary-row loading (load != 0:
 * rows after N_int move by +-load*dt per step), captured in a CUDA graph. */
int pd_run_adr(pd_ctx* ctx, int ct0, int nsteps, double load, void* stream);
/* Per-step body of the explicit drivers (Solve_Plate_Crack_Grow.cu:126-163,
 * Solve_Kalthoff_Winkler.cu:407-432) for nsteps steps: [quick_load(load)] +
 * Verlet + force (bond- or state-based by p->model) [+ contact when a
 * cylinder is installed], captured in a CUDA graph.  When dmg_every > 0 the
 * damage field is refreshed every dmg_every steps. */
int pd_run_explicit(pd_ctx* ctx, int nsteps, double load, int dmg_every, void* stream);

/* ---- quasi-static load stepping ---------------------------------------- */
/* No counterpart in the reference, which runs a fixed number of ADR steps
 * (Solve_Plate_Tensile.cu:106).  The residual of an iterate is |F + b|, the
 * 2-norm over the free (interior) nodes of internal plus body force. */
/* Residual at the current displacement: one force evaluation that leaves the
 * intact flags unchanged, then a fixed-order sum. */
int pd_residual(pd_ctx* ctx, double* norm, void* stream);
/* ADR steps ct0, ct0+1, ... (pd_run_adr's step, boundary rows held) in chunks
 * of check_every graph-captured steps, until the residual of an iterate is
 * <= tol or max_iters steps have run.  *iters receives the steps run and
 * *norm the last residual seen (that of the iterate the chunk's last step
 * started from; each step's force kernel reduces it beside the damping sums). */
int pd_adr_solve(pd_ctx* ctx, int ct0, int max_iters, int check_every, double tol, int* iters, double* norm,
                 void* stream);
typedef struct pd_load_step_stats {
    int32_t iters;      /* ADR steps run (probes included)                    */
    int32_t warm_used;  /* 0: plain start; k: the k-th candidate start        */
    int32_t probes;     /* candidates probed (rule 2)                         */
    int32_t pad_;
    double r_plain;     /* residual of the plain start (previous solution)     */
    double r_start;     /* residual of the start used                         */
    double r_final;     /* last residual seen                                 */
    double ms;          /* wall time of the whole increment (CUDA events)     */
} pd_load_step_stats;
/* One load increment: the boundary rows move by +-delta (kernel_quick_load's
 * rows), the ADR state restarts (half-step velocity and old force zero, step
 * index 0), and ADR runs until the residual is <= tol_rel times the plain
 * start's.  dev_du holds ncand (0..8) candidate increments on the device,
 * each N_int x increments then N_int y increments; a candidate start is the
 * previous solution plus the candidate.  Rule 1: a candidate whose start has
 * a larger residual than the plain start (the previous solution) is dropped;
 * with none left the plain start is used.  Rule 2: of several admissible
 * candidates, the one with the smallest starting residual is used when
 * probe_iters is 0; otherwise each runs probe_iters ADR steps and the one
 * with the lowest residual after them continues from where its probe ended
 * (the starting residual says little about how fast ADR converges: smooth
 * errors have small residuals and decay slowly).  The converged answer is the
 * plain method's in every case: all starts stop at the same residual. */
int pd_load_step(pd_ctx* ctx, double delta, const double* dev_du, int ncand, int probe_iters, double tol_rel,
                 int max_iters, int check_every, pd_load_step_stats* out, void* stream);

/* ---- learned warm start (per-node MLP on the tensor cores) --------------- */
/* No reference counterpart.  8 -> 128 -> 128 -> 128 -> 2, GELU on the hidden
 * layers, 34,434 parameters: BF16 operands of tcgen05.mma with FP32
 * accumulation; FP32 master parameters and Adam state for training.  Flat
 * parameter order (FP32, row-major [out][in]): W1[128][8], b1[128],
 * W2[128][128], b2[128], W3[128][128], b3[128], W4[2][128], b4[2].  Inputs
 * are BF16 rows of 16 (8 features, 8 zeros); outputs FP32 rows of 2. */
typedef struct pd_mlp pd_mlp;
pd_mlp* pd_mlp_create(int64_t max_rows, int* status);  /* rows per forward/backward pass */
int pd_mlp_destroy(pd_mlp* net);
int pd_mlp_num_params(void);
/* set (also resets the Adam state) / get the FP32 master parameters */
int pd_mlp_set_params(pd_mlp* net, const float* host, int64_t count);
int pd_mlp_get_params(pd_mlp* net, float* host, int64_t count);
/* y[M][2] = net(x[M][16]) (device pointers, x 16-byte and y 8-byte aligned;
 * 1 <= M <= 2^31 - 129, else PD_ERR_ARG): one persistent kernel runs the four
 * layers per 128-row tile with the weights resident in shared memory and the
 * activations kept on chip; weights and input tiles arrive by TMA (tensor
 * maps encoded per call; PD_ERR_CUDA if the driver cannot encode them). */
int pd_mlp_forward(pd_mlp* net, const void* dev_x, int64_t M, float* dev_y, void* stream);
/* The same forward pass layer by layer (one tensor-core product per layer
 * over max_rows blocks, activations through device memory): a check of
 * pd_mlp_forward, whose outputs it equals bit for bit. */
int pd_mlp_forward_layers(pd_mlp* net, const void* dev_x, int64_t M, float* dev_y, void* stream);
/* Gradient of loss = sum over rows and outputs of (y - t)^2 / (2 M), t[M][2] on
 * the device, M <= max_rows; flat gradient to host_grad (may be NULL). */
int pd_mlp_grad(pd_mlp* net, const void* dev_x, const float* dev_t, int64_t M, float* host_grad, float* loss,
                void* stream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on that loss. */
int pd_mlp_train_step(pd_mlp* net, const void* dev_x, const float* dev_t, int64_t M, float lr, float* loss,
                      void* stream);
/* The tensor-core product on its own: d[M][N] = a[M][K] * b[N][K]^T (BF16 in,
 * FP32 out; a stored [K][M] when transpose_a); N = 16 or a multiple of 128. */
int pd_mlp_gemm(const void* dev_a, const void* dev_b, int64_t M, int64_t N, int64_t K, float* dev_d, int transpose_a,
                void* stream);
/* Self-check of the bounded device-side wait: the same product with the
 * iteration limit of the kernel's mbarrier wait set to spin_limit (<= 0: the
 * library's limit, ~0.3 s) and, with issue = 0, neither the products nor
 * their commit issued, so that the wait never completes.  The kernel then
 * gives up after spin_limit iterations, releases its tensor memory and
 * returns; the call reports PD_ERR_TIMEOUT and the CUDA context stays
 * usable.  No counterpart in the reference (no tensor-core code). */
int pd_mlp_gemm_wait_check(const void* dev_a, const void* dev_b, int64_t M, int64_t N, int64_t K, float* dev_d,
                           int transpose_a, long long spin_limit, int issue, void* stream);
/* Features of the free nodes for a load increment (BF16 [N_int][16], 8
 * features, 8 zeros): previous displacement / U (x, y), increment / U,
 * damage, loaded-edge flag, and the history of the previous increment
 * (pd_warm_record): its departure from proportionality per unit load (x, y,
 * times 65536) and the damage it added (zeros without a history).  U is the
 * accumulated boundary displacement before the increment. */
int pd_warm_features(pd_ctx* ctx, double U, double delta, void* dev_x, void* stream);
/* The increment just solved becomes the history of the next prediction:
 * dev_u_prev (2*N_int: x then y) and dev_dmg_prev (N_int) hold the free
 * nodes' displacement and damage before it, U_prev the accumulated boundary
 * displacement before it.  Stored in the context: per node
 * ((u - u_prev) - u_prev delta / U_prev) / U_prev per component (the
 * departure of the increment from the proportional, secant, one per unit
 * load) and dmg - dmg_prev (the damage is brought up to date first).
 * U_prev <= 0 clears the history. */
int pd_warm_record(pd_ctx* ctx, double U_prev, double delta, const double* dev_u_prev, const double* dev_dmg_prev,
                   void* stream);
/* Candidate increments for pd_load_step (ncand = 2): dev_du[0 .. 2*N_int) =
 * u * delta / U + U * (h + net(features) / 65536), dev_du[2*N_int ..
 * 4*N_int) = u * delta / U.  The skip term is the proportional (secant)
 * increment, exact for a linear response loaded proportionally from rest; h
 * is the recorded history (pd_warm_record: the previous increment's
 * departure from proportionality per unit of accumulated boundary
 * displacement, zero without a history), and the network predicts how that
 * departure changes from one increment to the next, from the local state and
 * the history; it is trained on converged states of loadings through crack
 * advances (the increments in which a crack advanced left out).
 * smooth_passes > 0 (bond-based contexts): the correction U * net / 65536 is
 * first averaged that many times over each free node's intact family
 * (prescribed rows count as zero), which removes the node-to-node rounding
 * noise of the BF16 network that the residual amplifies. */
int pd_warm_predict(pd_ctx* ctx, pd_mlp* net, double U, double delta, int smooth_passes, double* dev_du,
                    void* stream);

/* ---- batches of specimens ----------------------------------------------- */
/* No counterpart in the reference, which solves one plate per process.  A
 * batch packs many 2-D bond-based plates of the crack-plate layout
 * (Coord.cu:34-45: nx*ny interior nodes, then 3 boundary rows above and 3
 * below) into one context and solves them together with the ADR step of
 * solve_plate_tensile (Solve_Plate_Tensile.cu:106-131), one launch per phase
 * for all specimens. */
typedef struct pd_specimen {
    int32_t nx, ny;       /* interior nodes per row, interior rows (>= 4 each) */
    double emod;          /* Young's modulus: sets bc and the ADR mass (Base.cuh:135, :150) */
    double critical_s;    /* critical stretch s0                               */
    double crack_len;     /* centred pre-crack length (0: none), kernel_set_crack_2D */
    double crack_theta;   /* pre-crack angle in radians                         */
    double load_scale;    /* boundary rows move by +-load_scale*load*dt per step */
} pd_specimen;
/* Builds the batch from shared parameters (dx, dt, thick, pratio, delta, MN,
 * mode: a 2-D bond-based pd_params, e.g. from pd_params_derive) and count
 * specimens: family (each specimen only with itself), surface correction,
 * per-specimen pre-crack, bond arrays.  Every specimen keeps its own
 * coordinate frame, so its coefficients and forces are those of the same
 * plate set up alone.  Node layout: specimen k's interior nodes start at
 * interior_offsets[k] (a multiple of 32; rows after its nx*ny nodes up to the
 * next offset are bond-less padding), its 6*nx boundary nodes at
 * N_int + boundary_offsets[k] (pd_batch_info).  Returns NULL and *status on
 * failure. */
pd_ctx* pd_batch_create(const pd_params* base, const pd_specimen* spec, int count, int* status);
/* count, and when non-NULL the count+1 interior and boundary offsets. */
int pd_batch_info(const pd_ctx* ctx, int* count, int64_t* interior_offsets, int64_t* boundary_offsets);
/* pd_run_adr for every specimen of a batch: each specimen has its own damping
 * coefficient (cal_cn over its own nodes) and ADR mass; boundary rows move by
 * +-load_scale*load*dt per step.  Three launches per step, CUDA graphs. */
int pd_batch_run_adr(pd_ctx* ctx, int ct0, int nsteps, double load, void* stream);
/* The count per-specimen damping coefficients of the last step. */
int pd_batch_get_cn(pd_ctx* ctx, double* cn, void* stream);

/* ---- launch shape of the bond-force kernels ------------------------------ */
/* Threads per block (128, 256, 512), warp-to-slice order (0: grid-strided,
 * 1: one contiguous run of slices per warp), grid size in waves of resident
 * blocks (1..8) and warps per slice (split: 1, 2, 4, 8; bond kernels,
 * strided order only): with split > 1 the slots of a slice are shared by
 * that many warps and summed by the first in the one-warp order (2-D: slot
 * order; 3-D: blocks of 32 slots, each summed in slot order, then the block
 * sums in order), which multiplies the bonds in flight on small problems and
 * evens out the last wave on large 3-D ones.  The per-node force sums do not
 * depend on the shape; sums over the whole grid (the single-specimen ADR
 * damping coefficient, the impactor reaction) follow the block order and may
 * differ in the last bits.  Default 256 / 0 / 1 / 1.  The reference's two
 * mappings, thread per node (kernel_particle_force_2D, Force_Bond.cu:52-85)
 * and warp per node (kernel_bond_force_2D, :6-50), correspond to split 1 and
 * to the widest split.  On the compact layout the 3-D bond kernel and the
 * state-based passes take the block size (at most 256 for the state-based
 * passes) and the waves; their unit order is fixed (the 3-D state-based
 * force pass: quarter slices with four slot phases). */
int pd_set_launch(pd_ctx* ctx, int block, int chunked, int waves, int split);
int pd_get_launch(const pd_ctx* ctx, int* block, int* chunked, int* waves, int* split);
/* Per-bond storage of the force kernels.  PD_LAYOUT_RECORDS: per bond slot
 * one 48-byte record (bond-based: column, float reference vector, c0, l0, k2,
 * break threshold) or three 32-byte records (state-based), any geometry.
 * PD_LAYOUT_COMPACT: one template per offset class (bonds whose reference
 * vectors round to the same float vector, one class per lattice offset on
 * the reference's regular grids: float vector, |xf|^2, |xf|^2 - l0t^2 and the
 * class's smallest length l0t) and small per-slot records: bond-based 16
 * bytes (column, l0 - l0t with the class id, k2 / 2; in 3-D the sign of k2
 * marks bonds the y >= -0.04 guard spares); state-based the column, l0 - l0t
 * with the class id and the reference vector's distance from the class's in
 * representable doubles (2-D 16 + 8 bytes, 3-D 8 + 16 + 8), the bond
 * coefficients per class.  For problems with at most 255 classes per
 * specimen whose bond lengths differ from their class's smallest by a float
 * with a free low byte; pd_prepare returns PD_ERR_UNSUPPORTED when a problem
 * does not fit.  PD_LAYOUT_AUTO (default): compact where it fits, records
 * otherwise.  Both layouts give the reference's intact flags and forces to
 * the same bars; the forces of the two differ in the last bits (different
 * pair arithmetic).  No counterpart in the reference, whose bond arrays are
 * padded ELL (Memory.cu:38-43).  Changing the layout releases the prepared
 * arrays. */
#define PD_LAYOUT_AUTO 0
#define PD_LAYOUT_RECORDS 1
#define PD_LAYOUT_COMPACT 2
int pd_set_force_layout(pd_ctx* ctx, int layout);
/* The layout prepared (PD_LAYOUT_AUTO: none yet). */
int pd_get_force_layout(const pd_ctx* ctx, int* layout);
/* Times the bond-force kernel (reps launches per shape, at the current
 * displacements) over the shapes above (24 with split 1: 1, 2, 4 or 8 waves;
 * 12 more with split 2 and 4; a 3-D compact context only the 12 strided
 * one-warp shapes) and keeps the fastest; *best_ms receives its time per
 * launch.  Intact flags and forces are restored, so a run continues exactly
 * as without the call.  Bond-based contexts only. */
int pd_autotune(pd_ctx* ctx, int reps, double* best_ms, void* stream);

/* ---- step profile --------------------------------------------------------- */
/* Runs nsteps steps of the ADR loop (kind 0: pd_run_adr, or pd_batch_run_adr
 * on a batch) or of the explicit loop (kind 1: pd_run_explicit without
 * damage passes) starting at step index ct0, launched directly rather than
 * from graphs, with CUDA events on the launch stream around each step's
 * force kernel(s) and around each whole step.  *force_ms and *step_ms receive
 * the averages per step.  The state advances as in those loops. */
int pd_profile_steps(pd_ctx* ctx, int kind, int ct0, int nsteps, double load, double* force_ms, double* step_ms,
                     void* stream);

/* ---- drivers (Solve_*.cuh:17-19) --------------------------------------- */
typedef struct pd_result {
    int64_t N, N_int, B;
    double setup_ms;      /* neighbour + setup passes          */
    double loop_ms;       /* time-step loop (CUDA events)      */
    double bond_updates_per_s;
} pd_result;
/* solve_plate_tensile (Solve_Plate_Tensile.cu:30-138) with dx (<=1e-8 -> 0.01).
 * Host arrays ux, uy, dmg (N_int each) receive the final fields when non-NULL. */
int pd_solve_plate_tensile(double dx, int nt, double* ux, double* uy, double* dmg, pd_result* res);
/* solve_plate_crack_grow (Solve_Plate_Crack_Grow.cu:167-308). */
int pd_solve_plate_crack_grow(double dx, int nt, double* ux, double* uy, double* dmg, pd_result* res);
/* solve_kalthoff_winkler (Solve_Kalthoff_Winkler.cu:268-441); the reference
 * runs nt=0 steps, this takes nt. Arrays hold N entries (see res->N). */
int pd_solve_kalthoff_winkler(double dx, int nt, double* ux, double* uy, double* uz, double* dmg,
                              int64_t cap, pd_result* res);

/* ---- output ------------------------------------------------------------ */
/* save_disp_gpu / save_disp_cpu (Save.cu:6-60): one line per interior node,
 * "ux uy dmg" (uz == NULL) or "ux uy uz dmg", each value as std::ostream
 * prints a double by default (%g, 6 significant digits). */
int pd_write_disp_txt(const char* path, int64_t n, const double* ux, const double* uy, const double* uz,
                      const double* dmg);
/* save_kw_gpu / save_kw_cpu (Save.cu:62-140): the first z layer of the
 * notched slab in grid order (p->nx x p->ny), notch cells of the upper half
 * written as "nan nan 0 nan"; n is the number of node values available. */
int pd_write_kw_txt(const char* path, const pd_params* p, double rad, int64_t n, const double* ux,
                    const double* uy, const double* uz, const double* dmg);
/* The same writers fed from a context (its N_int interior nodes). */
int pd_save_disp(pd_ctx* ctx, const char* path, void* stream);
int pd_save_kw(pd_ctx* ctx, double rad, const char* path, void* stream);
/* Binary snapshot of the simulation state: displacement, velocity,
 * acceleration, force, body force, ADR half-step velocity and old force, damage
 * and dilatation (N doubles per component), the intact flags (B int32), the ADR
 * damping coefficient and the impactor.  No reference counterpart (its output
 * is text only).  Loading needs a context with the same set-up (N, N_int, B,
 * dim, model); a run continued from a loaded snapshot repeats the saved run
 * bit for bit. */
int pd_snapshot_save(pd_ctx* ctx, const char* path, void* stream);
int pd_snapshot_load(pd_ctx* ctx, const char* path, void* stream);
/* Number of broken bonds (intact flag 0) over the whole family, counted on
 * the device; the caller's copy is one integer.  No counterpart in the
 * reference, whose drivers read the fail array back to the host. */
int pd_count_broken(pd_ctx* ctx, int64_t* count, void* stream);
/* Crack tip from the damage field: the interior node with the largest x among
 * those with dmg > threshold (lowest index among ties); tip_xy receives its
 * reference coordinates, NaN when no node is damaged.  The reference's tracker
 * (commented out, Solve_Plate_Crack_Grow.cu:150-162) scans one row for dmg > 0.38. */
int pd_crack_tip(pd_ctx* ctx, double threshold, double* tip_xy, void* stream);

/* ---- diagnostics ------------------------------------------------------- */
/* NaN/Inf scan of displacement and force; PD_ERR_NONFINITE if any. */
int pd_check_finite(pd_ctx* ctx, void* stream);
/* Number of GPU kernels this context has launched (for launch accounting). */
int64_t pd_kernel_launches(const pd_ctx* ctx);
/* Allocation-free sum of n doubles of a device array into *dev_result (a
 * device pointer), in a fixed summation order.  No counterpart in the
 * reference: for callers that cannot allocate device memory (a component
 * that owns the allocator, a foreign-function caller without a context, a
 * path that must not allocate).  Needs no context and allocates nothing: the
 * block partial sums use a 64 KiB array in the library's own device memory,
 * which every GPU that loads the library keeps until exit.  n is at most
 * 33,554,432 (8,192 blocks of 4,096 elements); larger n returns PD_ERR_ARG.
 * The first call in each CUDA context (one per device for runtime-API
 * callers; a context rebuilt by cudaDeviceReset or a driver-API caller's own
 * context counts as a new one) looks the array's address up
 * (cudaGetSymbolAddress) and must come before any stream capture that
 * contains this call.  All calls share the array: calls that overlap on the
 * GPU (different streams, no ordering between them) race and may return
 * wrong sums. */
int pd_reduce_sum_static(const double* dev_x, int64_t n, double* dev_result, void* stream);

/* FP64 FMA issue rate of the current device in 1e9 FMA/s (dependent-chain
 * microbenchmark, best of 3): the denominator of the FP64 roofline. */
int pd_probe_fp64(double* gfma_per_s);

/* Self-check of the division recipe the update kernels use for a divisor
 * with a known reciprocal (density, ADR mass, the ADR update's 2 + cn dt, the
 * state-based 1/m): n / d formed from y = 1 / d by two FMA corrections
 * (Markstein's correctly rounded division) against the IEEE division, on
 * count device pairs dev_n[i] / dev_d[i].  Writes the number of quotients
 * whose bit patterns differ to *dev_mismatches (a device counter).  No
 * counterpart in the reference, whose kernels divide directly. */
int pd_check_division(const double* dev_n, const double* dev_d, int64_t count, unsigned long long* dev_mismatches,
                      void* stream);

#ifdef __cplusplus
}
#endif
#endif /* PD_GB300_H */
