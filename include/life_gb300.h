/*
 * life_gb300.h -- C-ABI of the GB300 LIFE hot path.
 *
 * The LIFE reference (joconnor22/LIFE v1.0.3) has no plugin or FFI layer: its
 * boundary is the class interface that main() drives (reference
 * src/main.cpp:42-86) -- GridClass() (src/Grid.cpp:1232), ObjectsClass(GridClass&)
 * (src/Objects.cpp:1589), GridClass::solver() (src/Grid.cpp:25), the
 * IBMBodyClass constructors (src/IBMBody.cpp:27,45,79) and the restart
 * readers/writers (src/Grid.cpp:1072-1229, src/Objects.cpp:979-1371). Each entry
 * point below replaces one of those; the comment on each names which.
 *
 * Conventions
 *   - Plain C types only; every function returns an int status (LIFE_OK = 0).
 *     life_last_error() gives the message the reference would have printed
 *     through ERROR() before exit(99) (reference inc/Utils.h:72-77).
 *   - Device memory is owned by the library; host buffers by the caller.
 *   - Field buffers use the reference's host layout: site id = i*Ny + j
 *     (y fastest), populations f[id*9 + v], velocity u[id*2 + d].
 *   - A LifeCase handle is not thread-safe; distinct handles are independent.
 */
#ifndef LIFE_GB300_H
#define LIFE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LIFE_ABI_VERSION 1

/* Status codes */
enum {
    LIFE_OK = 0,
    LIFE_ERR_INVALID = 1,       /* bad argument or unsupported case option */
    LIFE_ERR_CUDA = 2,          /* a CUDA runtime call failed */
    LIFE_ERR_NAN = 3,           /* "Simulation blew up" (reference src/Grid.cpp:573-581) */
    LIFE_ERR_SUBITER = 4,       /* subiteration cap hit (src/Objects.cpp:58-59) */
    LIFE_ERR_SUPPORT = 5,       /* support buffer overflow (src/IBMNode.cpp:171-172) */
    LIFE_ERR_GEOMETRY = 6,      /* geometry.config / body construction errors */
    LIFE_ERR_DEFLECT = 7,       /* static pre-deflection cap (src/FEMBody.cpp:427-428) */
    LIFE_ERR_NOMEM = 8,         /* device allocation failed */
    LIFE_ERR_TIMEOUT = 9,       /* a bounded device wait gave up */
    LIFE_ERR_BUSY = 10          /* serving queue full / slot not ready */
};

/* eLatType (reference inc/defs.h:51); LIFE_FLUID on a wall means periodic. */
enum { LIFE_FLUID = 0, LIFE_WALL = 1, LIFE_VELOCITY = 2, LIFE_FREESLIP = 3,
       LIFE_PRESSURE = 4, LIFE_CONVECTIVE = 5 };
/* eProfileType (reference inc/defs.h:52); UNIFORM = PROFILE undefined. */
enum { LIFE_PROFILE_UNIFORM = -1, LIFE_PROFILE_PARABOLIC = 0, LIFE_PROFILE_SHEAR = 1,
       LIFE_PROFILE_BOUNDARY_LAYER = 2 };
/* Population storage/arithmetic form on the GPU. */
enum { LIFE_PREC_F64 = 0, LIFE_PREC_F32 = 1, LIFE_PREC_F16 = 2 };
/* geometry.config keywords (reference src/Objects.cpp:374-382) */
enum { LIFE_BODY_CIRCLE = 0, LIFE_BODY_FILAMENT = 1 };

/* Every value of the reference's params.h that the solver reads
 * (reference inc/params.h:26-110). Switches that are #define'd or not in
 * params.h become has_* flags. include/life_params_pack.h fills this struct
 * from a params.h at compile time. */
typedef struct LifeCaseParams {
    int32_t Nx, Ny;
    double height_p, rho_p, nu_p, omega;
    double ux0_p, uy0_p;
    double gravityX, gravityY, dpdx, dpdy;
    int32_t wall_left, wall_right, wall_bottom, wall_top;
    int32_t profile;
    double uxInlet_p, uyInlet_p;
    double alpha, delta;          /* Newmark */
    double relaxMax, subTol;      /* FSI coupling */
    int32_t central_moments;
    int32_t has_inlet_ramp;  double inlet_ramp;
    int32_t has_womersley;   double womersley;
    int32_t uni_epsilon, ordered;
    int32_t has_initial_deflect; double initial_deflect;
    int32_t nSteps, tinfo, tVTK, tRestart;
    double ref_nu, ref_rho, ref_P, ref_L, ref_U;
    int32_t precision;            /* LIFE_PREC_* (GPU only; not a params.h value) */
    int32_t reserved[7];
} LifeCaseParams;

/* One geometry.config line (reference input/geometry.config:8-13):
 *   CIRCLE   NUMBER ID X Y DX DY RADIUS
 *   FILAMENT NUMBER ID X Y DX DY LENGTH HEIGHT ANGLE FLEXIBLE|RIGID
 *            N_ELEMENTS|CONFORMING CLAMPED|SUPPORTED DENSITY YOUNG_MODULUS */
typedef struct LifeBodyDesc {
    int32_t kind;         /* LIFE_BODY_CIRCLE / LIFE_BODY_FILAMENT */
    int32_t number;       /* NUMBER of bodies in this line */
    int32_t id;           /* STARTID */
    int32_t flexible;     /* FILAMENT: 1 FLEXIBLE, 0 RIGID */
    int32_t n_elements;   /* FILAMENT: element count, 0 = CONFORMING */
    int32_t clamped;      /* FILAMENT: 1 CLAMPED, 0 SUPPORTED */
    double x, y, dx, dy;  /* start position and spacing (physical units) */
    double radius;        /* CIRCLE */
    double length, height, angle_deg;  /* FILAMENT */
    double rho, E;        /* FILAMENT density and Young's modulus */
} LifeBodyDesc;

/* Sizes of a created case (after marker de-overlap). */
typedef struct LifeCaseInfo {
    int32_t Nx, Ny;
    int32_t n_bodies, n_markers, n_flex, sim_dofs;
    int32_t precision;
    int32_t t;                 /* current time step */
    double Dx, Dt, Dm, Drho, tau, nu, c_s;
    size_t device_bytes;       /* device memory held by the case */
} LifeCaseInfo;

/* Device-side status flags and per-step diagnostics. */
typedef struct LifeStatus {
    int32_t code;              /* first error seen (LIFE_ERR_*), 0 if none */
    int32_t t;                 /* time step at which it was raised */
    int32_t last_subits;       /* subiterations taken in the last step */
    int32_t last_nr_its;       /* NR iterations of body 0 in the last subiteration */
    double last_subres;        /* FSI residual reached */
    double relax;              /* current Aitken factor */
} LifeStatus;

typedef struct LifeCase LifeCase;

/* Version of this ABI (LIFE_ABI_VERSION). */
int life_abi_version(void);

/* Message for the last error raised on this thread (never NULL). */
const char* life_last_error(void);

/* Replaces GridClass::GridClass (src/Grid.cpp:1232-1289) followed by
 * ObjectsClass::ObjectsClass (src/Objects.cpp:1589-1624): builds the lattice,
 * the type map and inlet profiles (initialiseGrid, src/Grid.cpp:916-1062), the
 * IBM bodies from the geometry lines (geometryReadIn, src/Objects.cpp:324-488;
 * IBMBodyClass ctors src/IBMBody.cpp:45-135), removes overlapping markers
 * (src/Objects.cpp:867-938) and runs initialiseObjects (src/Objects.cpp:941-961).
 * All state is then uploaded to device 0 (or the current device). */
int life_case_create(const LifeCaseParams* params, const LifeBodyDesc* bodies,
                     int32_t n_bodies, LifeCase** out);

/* Releases the case and its device memory. */
int life_case_destroy(LifeCase* c);

/* Replaces nsteps iterations of the main loop's grid.solver()
 * (src/main.cpp:70-73, GridClass::solver src/Grid.cpp:25-33). Asynchronous with
 * respect to the host unless an error must be reported; t advances by nsteps. */
int life_case_step(LifeCase* c, int32_t nsteps);

/* Blocks until all queued work of the case has finished; returns the device
 * status code (LIFE_ERR_SUBITER etc.) if one was raised. */
int life_case_sync(LifeCase* c);

int life_case_info(const LifeCase* c, LifeCaseInfo* info);
int life_case_status(LifeCase* c, LifeStatus* st);

/* Copies the reference's grid state after the current step into host buffers
 * in the reference layout (any pointer may be NULL to skip it): rho[Nx*Ny],
 * u[Nx*Ny*2], f[Nx*Ny*9], force_ibm[Nx*Ny*2]. These are exactly the arrays
 * GridClass::writeRestart dumps (src/Grid.cpp:1191-1222). */
int life_case_get_fields(LifeCase* c, double* rho, double* u, double* f, double* force_ibm);

/* Replaces GridClass::readRestart (src/Grid.cpp:1072-1160): loads rho, u,
 * force_ibm and f (reference layout) and sets the time step to t. */
int life_case_set_fields(LifeCase* c, int32_t t, const double* rho, const double* u,
                         const double* f, const double* force_ibm);

/* Marker arrays in global marker order (iNode order after de-overlap):
 * pos/vel/force [n*2], epsilon/ds [n], body_index [n]. NULL skips a field. */
int life_case_get_markers(LifeCase* c, double* pos, double* vel, double* force,
                          double* epsilon, double* ds, int32_t* body_index);
/* Body table: reference body IDs, flexible flags and marker counts. */
int life_case_get_bodies(LifeCase* c, int32_t* ids, int32_t* flexible, int32_t* n_markers,
                         int32_t* n_fem_nodes);

/* Body shapes and marker lists, as ObjectsClass::writeVTK walks them
 * (src/Objects.cpp:738-830): kind[n_bodies] (LIFE_BODY_CIRCLE or
 * LIFE_BODY_FILAMENT; a circle's outline is closed) and, body after body, the
 * global index of each of the body's markers in its node order
 * (marker_index[n_markers]). Either pointer may be NULL. */
int life_case_get_body_nodes(LifeCase* c, int32_t* kind, int32_t* marker_index);

/* The arrays GridClass::writeVTK writes to Results/VTK/Fluid.<t>.vti
 * (src/Grid.cpp:790-913) for the current state, in VTK point order (x
 * fastest: point j*Nx + i): density[Nx*Ny] = rho*Drho, pressure[Nx*Ny] =
 * ref_P + (rho - rho_p/Drho) c_s^2 Dm / (Dx Dt^2) and velocity[Nx*Ny*3] =
 * (ux, uy, 0) Dx/Dt, each with the reference's operation order. Formed on
 * the device, in the device's own site order; any pointer may be NULL. */
int life_case_get_vtk_fields(LifeCase* c, double* density, double* pressure, double* velocity);

/* Support table of every marker (IBMNodeClass::supp, reference
 * inc/IBMNode.h:69-70): count nsupp[n], lattice indices si/sj[n*9] and delta
 * weights sd[n*9], as findSupport left them (src/IBMNode.cpp:139-179). */
int life_case_get_support(LifeCase* c, int32_t* nsupp, int32_t* si, int32_t* sj, double* sd);

/* Epsilon weights of the implicit IBM for one marker set, on device buffers
 * the caller owns (ObjectsClass::computeEpsilon, src/Objects.cpp:264-311):
 * solves A eps = 1 with A_ij = (sum_s d_i(s) delta(x_j - s)) ds_j. Inputs are
 * device pointers pos[n*2], nsupp[n], si/sj/sd[n*9], ds[n] in lattice units
 * (pos in physical units, Dx the lattice spacing); eps[n] is written. Runs on
 * `stream` (a cudaStream_t, NULL for the default stream) and returns when the
 * result is ready. Allocates the n x n system for the duration of the call. */
int life_ibm_epsilon(const double* pos, const int32_t* nsupp, const int32_t* si, const int32_t* sj,
                     const double* sd, const double* ds, int32_t n, double Dx, double* eps, void* stream);

/* life_ibm_epsilon without any device allocation. No counterpart in the
 * reference (which has no GPU memory to manage): it exists for callers that
 * cannot call cudaMalloc, because their device memory all comes from another
 * allocator's pool or because cudaMalloc/cudaFree's implicit device
 * synchronisation is not allowed where they run. The n x n system lives in a
 * library-owned static device array sized for at most 256 markers (516 KiB,
 * held on every GPU that loads the library until exit); larger n is rejected
 * with LIFE_ERR_INVALID. All calls share that array, so calls that overlap on
 * the GPU race; the caller must order them. The first call on each device
 * looks up the array's device address, and should come before any stream
 * capture on that device; the address is kept until exit, so the library must
 * not be used on a device across a cudaDeviceReset. Unlike life_ibm_epsilon
 * the call does not wait: it queues the solve on `stream` and returns, and
 * eps is ready once that stream reaches this point. Same arguments and result
 * as life_ibm_epsilon. */
int life_ibm_epsilon_noalloc(const double* pos, const int32_t* nsupp, const int32_t* si, const int32_t* sj,
                             const double* sd, const double* ds, int32_t n, double Dx, double* eps,
                             void* stream);

/* FEM state of flexible body k (in body order): each array has 3*n_fem_nodes
 * entries, or n_el / n_node entries for the element and node arrays.
 * The set mirrors FEM.restart (src/Objects.cpp:1289-1362). */
int life_case_get_fem(LifeCase* c, int32_t k, double* U, double* Udot, double* Udotdot,
                      double* U_n, double* U_nm1, double* R_k, double* el_L,
                      double* el_angle, double* node_pos, double* node_angle);
int life_case_get_relax(LifeCase* c, double* relax);

/* Restart readers for bodies, the counterpart of life_case_set_fields for
 * ObjectsClass::readRestart (src/Objects.cpp:979-1203). set_markers loads
 * marker pos/vel/force [n*2] in global marker order (NULL skips a field) and
 * then recomputes every marker's support and ds and the epsilon weights
 * (src/Objects.cpp:1181-1192). set_fem loads flexible body k's FEM.restart
 * arrays (3*n_fem_nodes DOF vectors, n_el element lengths/angles, n_node
 * positions [n*2] and angles; NULL keeps the case's own) and recomputes the
 * element transforms (src/Objects.cpp:1195-1200). set_relax sets the Aitken
 * factor stored in FEM.restart. A restart loads fields, markers, FEM bodies
 * and relax, in any order, before the next step. */
int life_case_set_markers(LifeCase* c, const double* pos, const double* vel, const double* force);
int life_case_set_fem(LifeCase* c, int32_t k, const double* U, const double* Udot, const double* Udotdot,
                      const double* U_n, const double* U_nm1, const double* R_k, const double* el_L,
                      const double* el_angle, const double* node_pos0, const double* node_pos,
                      const double* node_angle0, const double* node_angle);
int life_case_set_relax(LifeCase* c, double relax);
/* Undeformed node positions [n*2] and angles [n] of flexible body k (the pos0
 * and angle0 columns of FEM.restart). */
int life_case_get_fem0(LifeCase* c, int32_t k, double* node_pos0, double* node_angle0);

/* Scalar observables computed on the device without copying the field:
 * max |u| over the lattice with a NaN check (GridClass::writeInfo,
 * src/Grid.cpp:562-588) and the total IBM force (writeTotalForces,
 * src/Objects.cpp:518-528). */
int life_case_max_velocity(LifeCase* c, double* max_vel, int32_t* has_nan);
int life_case_total_force(LifeCase* c, double* fx, double* fy);

/* Observables recorder: the rows ObjectsClass::writeTotalForces and
 * ObjectsClass::writeTips append every tinfo steps (src/Objects.cpp:491-594,
 * called from Utils::writeInfo, src/Utils.cpp:120-137), gathered on the device
 * inside the step graph, with no host synchronisation per row.
 * life_case_record(c, every, capacity) records a row for every step t with
 * t % every == 0 (and one for the current state at once, as the reference
 * writes one before its first step), into a device buffer of `capacity` rows;
 * every <= 0 removes the recorder. A row holds Fx, Fy (the reference's total
 * force: minus the sum over markers of force * 1.0 * eps * ds * forceScale, in
 * marker order) and, for each flexible body in body order, the x, y, vx, vy
 * of its last marker (the reference's tip). Call it between steps.
 * life_case_records copies the rows recorded so far (oldest first) into
 * t[n_rows] and rows[n_rows * n_cols], and empties the buffer; rows that found
 * it full are counted in *dropped. Fails with LIFE_ERR_INVALID when more than
 * max_rows rows are waiting. With t and rows both NULL it only reports
 * n_rows, n_cols and dropped and leaves the rows in place. */
int life_case_record(LifeCase* c, int32_t every, int32_t capacity);
int life_case_records(LifeCase* c, int32_t max_rows, int32_t* n_rows, int32_t* n_cols, int32_t* t,
                      double* rows, int32_t* dropped);

/* Measurement hook (no counterpart in the reference, which only prints an
 * MLUPS figure from wall-clock time, src/Grid.cpp:594-610): runs nsteps steps
 * like life_case_step and returns the device time of the whole range and the
 * mean device time of the interior lattice kernel, both from CUDA events
 * recorded on the case's stream, and the number of kernels launched. */
int life_case_bench_steps(LifeCase* c, int32_t nsteps, double* total_ms, double* interior_ms,
                          int32_t* launches);

/* ---- Batched ensembles (no counterpart in the reference, which runs one case
 * per process). A batch steps many independent cases of uneven lattice size,
 * body count and collision model together: the interior stream-collide of all
 * cases runs in one persistent launch over per-case tile ranges, the rest of
 * each case's step runs on the case's own stream, and one batch step is a
 * replayed CUDA graph (a case's FSI subiteration loop is a conditional WHILE
 * node in it). Each case computes exactly what it computes alone. All cases
 * must use the same population storage form. */
typedef struct LifeBatch LifeBatch;

typedef struct LifeBatchInfo {
    int32_t n_cases, precision;
    int64_t sites;             /* lattice sites over all cases */
    int32_t tile_w, tile_h;    /* tile shape of the batched interior launch */
    int32_t tiles, grid;       /* tiles over all cases, persistent CTAs */
    int32_t kernel_nodes;      /* kernel nodes of one step graph (loop bodies once) */
    size_t device_bytes;       /* device memory held by the cases */
} LifeBatchInfo;

/* Creates n_cases cases: params[k] with n_bodies[k] consecutive entries of
 * `bodies` (as life_case_create). */
int life_batch_create(const LifeCaseParams* params, const LifeBodyDesc* bodies, const int32_t* n_bodies,
                      int32_t n_cases, LifeBatch** out);
int life_batch_destroy(LifeBatch* b);
/* Advances every case by nsteps steps; returns the first case's device status
 * error (with the case index in the message) if one was raised. */
int life_batch_step(LifeBatch* b, int32_t nsteps);
int life_batch_sync(LifeBatch* b);
/* Borrowed handle of case k for the life_case_get_* and status calls (the
 * batch keeps ownership; stepping it alone makes the batch recapture). */
int life_batch_case(LifeBatch* b, int32_t k, LifeCase** out);
int life_batch_info(LifeBatch* b, LifeBatchInfo* info);
/* Tile shape of the batched interior launch: tile_w in 32..256 (multiple of
 * 32, one CTA row), tile_h rows per tile. */
int life_batch_set_tile(LifeBatch* b, int32_t tile_w, int32_t tile_h);
/* Times the batched interior kernel for tile_w in {64,128,256} x tile_h in
 * {1,2,4,8} on this batch and keeps the fastest; returns it and its time. */
int life_batch_autotune(LifeBatch* b, int32_t* tile_w, int32_t* tile_h, float* best_ms);
/* Mean device time of the batched interior kernel alone (measurement hook). */
int life_batch_interior_ms(LifeBatch* b, int32_t reps, float* ms);
/* Runs nsteps batch steps between CUDA events on the batch stream and returns
 * their device time and the kernel nodes per step graph (measurement hook). */
int life_batch_bench_steps(LifeBatch* b, int32_t nsteps, double* total_ms, int32_t* kernels_per_step);

/* ---- Serving (no counterpart in the reference). A server owns a thread that
 * admits submitted solves in arrival order while their estimated device
 * footprint fits hbm_budget, keeps their state on the device, and steps all
 * admitted requests together as one batch per storage form, in rounds of at
 * most steps_per_round steps; the active set is regrouped whenever a request
 * is admitted or finishes (continuous batching). A finished request keeps its
 * state on the device (counted against the budget) until it is taken or
 * released. Each request computes exactly what it computes alone. The server
 * calls are thread-safe. */
typedef struct LifeServer LifeServer;

typedef struct LifeServerConfig {
    size_t hbm_budget;         /* bytes the admitted requests may hold */
    int32_t max_active;        /* requests stepped together at most (0: no limit) */
    int32_t steps_per_round;   /* steps per scheduling round (0: 200) */
} LifeServerConfig;

enum { LIFE_REQ_QUEUED = 0, LIFE_REQ_RUNNING = 1, LIFE_REQ_DONE = 2, LIFE_REQ_FAILED = 3 };

typedef struct LifeRequestInfo {
    int32_t state;             /* LIFE_REQ_* */
    int32_t error;             /* LIFE_ERR_* of a failed request */
    int32_t steps_done, steps;
    double submit_s, start_s, done_s;  /* server clock, seconds since creation */
    size_t device_bytes;
    int64_t sites;
} LifeRequestInfo;

typedef struct LifeServerStats {
    int64_t submitted, admitted, completed, failed;
    int32_t active, queued;
    size_t bytes_in_use, bytes_peak;
    int64_t rounds, regroups;
    double site_steps;         /* lattice-site updates done */
    double busy_s;             /* server-clock time with admitted work */
    double clock_s;            /* server clock now */
} LifeServerStats;

int life_server_create(const LifeServerConfig* cfg, LifeServer** out);
/* Queues a solve of nsteps steps of the case (params, bodies); returns its id. */
int life_server_submit(LifeServer* s, const LifeCaseParams* params, const LifeBodyDesc* bodies,
                       int32_t n_bodies, int32_t nsteps, int64_t* id);
int life_server_query(LifeServer* s, int64_t id, LifeRequestInfo* info);
/* Blocks until the request is done or failed (its error), or LIFE_ERR_TIMEOUT
 * after timeout_s seconds (negative: no limit). */
int life_server_wait(LifeServer* s, int64_t id, double timeout_s);
/* Hands a done request's case (device state) to the caller, who destroys it. */
int life_server_take(LifeServer* s, int64_t id, LifeCase** out);
/* Frees a done or failed request. */
int life_server_release(LifeServer* s, int64_t id);
int life_server_stats(LifeServer* s, LifeServerStats* st);
/* Blocks until nothing is queued or running (LIFE_ERR_TIMEOUT after timeout_s). */
int life_server_drain(LifeServer* s, double timeout_s);
/* Stops the thread (queued requests are dropped) and frees everything. */
int life_server_destroy(LifeServer* s);

/* Self-test of the library's division by a known reciprocal (used by the
 * FEM band solve): compares it with IEEE division on n seeded random operand
 * pairs on the device and returns the number of results that differ. */
int life_selftest_division(int64_t n, uint64_t seed, int64_t* mismatches);

/* Self-test of the device's correctly rounded trigonometry (the FEM element
 * angle and rotation): evaluates op 0 = sin(x), 1 = cos(x), 2 = atan2(y, x)
 * on the device for n host operands and writes the results to out[n]. */
int life_selftest_trig(int32_t op, int64_t n, const double* x, const double* y, double* out);

/* Measurement helper (no counterpart in the reference): the FP64 rate this
 * GPU sustains on independent fused multiply-add chains, in GFLOP/s (an FMA
 * counts two). It is the roofline denominator of the FP64 lattice kernels,
 * which the SM's FP64 unit bounds. Runs on the current device and waits. */
int life_measure_fp64_rate(double* gflops);

/* Parses geometry.config text with the reference's rules (leading '#' lines
 * skipped, whitespace tokens; src/Objects.cpp:338-458). Writes at most cap
 * descriptors, returns the number found in *n.
 * Besides CIRCLE and FILAMENT it reads one keyword of its own, added the way
 * the reference's README (README.md:36-40) describes, for canopies of stalks
 * of random length and stiffness:
 *   CANOPY NUMBER STARTID STARTX STARTY SPACING_X SPACING_Y LENGTH_MIN
 *          LENGTH_MAX HEIGHT ANGLE N_ELEMENTS|CONFORMING CLAMPED|SUPPORTED
 *          DENSITY_PER_LENGTH YOUNG_MIN YOUNG_MAX SEED
 * expands into NUMBER flexible FILAMENT descriptors (one body each, IDs from
 * STARTID, stalk k at START + k*SPACING): length L = LENGTH_MIN +
 * (LENGTH_MAX - LENGTH_MIN)*r, density DENSITY_PER_LENGTH*L, Young's modulus
 * (YOUNG_MIN*(YOUNG_MAX/YOUNG_MIN)^r')*(L*L*L), where r, r' are the stalk's
 * two draws of SplitMix64 seeded with SEED ((z >> 11) * 2^-53 per draw).
 * With a mass ratio m and a bending stiffness S = EI/(rho U^2 L^3) at fluid
 * density rho, inlet U, I = Dx H^3/12: DENSITY_PER_LENGTH = m rho / H and
 * Young's modulus = 12 S rho U^2 L^3 / (Dx H^3). */
int life_parse_geometry(const char* text, LifeBodyDesc* out, int32_t cap, int32_t* n);

#ifdef __cplusplus
}
#endif
#endif /* LIFE_GB300_H */
