/*
 * taichimps_gb300 — C ABI of the GB300 (sm_103a) granular-DEM contact path.
 *
 * Every entry point takes plain device pointers owned by the caller (the
 * library never allocates or frees caller memory), a stream, and returns an
 * int: TMPS_OK, or TMPS_ERR_BAD_ARG / TMPS_ERR_CUDA for a launch that could
 * not be made.  Launches are asynchronous on the given stream.  Errors found
 * on the device (a neighbor row that overflowed, a non-finite position, a box
 * driven non-positive) are OR-ed into the caller's `int32_t* status` word,
 * which the host reads when it synchronises anyway (rebuilds, output, the end
 * of a run) — the same places the reference raises.
 *
 * Layout (internal atom order; the neighbor build re-sorts atoms by cell):
 *   xr  double[n][4]  x, y, z, radius
 *   vm  double[n][4]  vx, vy, vz, mass
 *   om  double[n][4]  wx, wy, wz, moment of inertia 0.4*m*r*r
 *   f, torque  double[3][n]   (component-major)
 *   virial     double[6][n]   [xx, yy, zz, xy, xz, yz], optional
 *   nbr    int32[slots][n]    full neighbor list, slot-major
 *   shear  double[3][slots][n] per-slot shear, in the row atom's i->j sense
 *   touch  uint64[n]          bit k set while slot k is in contact
 *
 * Each declaration names the reference interface it replaces
 * (taichimps, path within the project, file:line).
 */
#ifndef TAICHIMPS_GB300_H
#define TAICHIMPS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    TMPS_OK = 0,
    TMPS_ERR_BAD_ARG = 1,
    TMPS_ERR_CUDA = 2,
    TMPS_ERR_TOO_LARGE = 3,  /* beyond the fixed scratch of tmps_nlist_build_noalloc */
};

/* Size limits of tmps_nlist_build_noalloc's built-in scratch. */
#define TMPS_NOALLOC_MAX_ATOMS 1048576
#define TMPS_NOALLOC_MAX_CELLS 200000

/* Bits of the device status word. */
enum {
    TMPS_STATUS_NLIST_OVERFLOW = 1,   /* a row needed more than `slots` entries */
    TMPS_STATUS_NONFINITE = 2,        /* a position became NaN/Inf */
    TMPS_STATUS_BOX_NONPOSITIVE = 4,  /* the servo drove a box length <= 0 */
    TMPS_STATUS_CELL_OVERFLOW = 8,    /* grid larger than the cell buffers */
};

/* Device-resident box: written by the host (tmps_box_set) or by the servo
 * kernel, read by every kernel.  Replaces the zero-dimensional box fields of
 * Domain (src/taichimps/domain.py:55-68, _sync_kernel :188-233). */
typedef struct tmps_box {
    double lo[3];
    double hi[3];
    double prd[3];
    double inv_prd[3];  /* 1/prd, kept beside prd so no kernel divides per thread */
    double h_rate[6];   /* box length rates [x, y, z, yz, xz, xy] */
    int32_t per[3];
    int32_t vremap;     /* remap v: partner velocity shift across images */
    /* neighbor grid, fixed at the last build */
    int32_t g[3];
    int32_t ncell;
    double csize[3];    /* lamda bin size 1/g */
    double hcell[3];    /* Cartesian bin size prd/g (follows the box) */
    /* box as it was before the last servo update (remap x reads it) */
    double old_lo[3];
    double old_prd[3];
    int32_t remap_pending;
    int32_t pad_;
} tmps_box;

/* Per-atom storage (pointers into caller memory). */
typedef struct tmps_atoms {
    int32_t n;
    int32_t pad_;
    double* xr;
    double* vm;
    double* om;
    double* f;
    double* torque;
    double* virial;     /* may be NULL */
    int32_t* tag;
    int32_t* uid;       /* insertion index of each internal slot */
    double* x0;         /* double[3][n]: positions at the last build */
    /* mixed-precision mirrors (may be NULL in the FP64 form) */
    float* pos32;       /* float[n][4]: offset from cell origin, radius */
    int32_t* cell32;    /* cell coordinate, cx | cy << 10 | cz << 20 */
    float* vel32;       /* float[n][4]: v, mass */
    float* om32;        /* float[n][4]: omega, v lo x (see the low words below) */
    float* f32;         /* float[3][n] contact force, mixed form */
    float* torque32;    /* float[3][n] */
    float* o0_32;       /* float[3][n]: offsets at the last build (mixed skin check) */
    double* rinv;       /* double[2][n]: 1/m, 1/I (fused FP64 step) */
    /* Low words of the mixed form's double-word state: value = hi + lo with
     * both FP32 (~48-bit significand).  pos32lo = (offset lo, radius lo);
     * the velocity and angular velocity low words are packed so that the
     * update kernel rewrites no per-build constant beside them: v lo x in
     * om32's fourth lane, lo32 = (v lo y, v lo z, omega lo x, omega lo y),
     * wlz32 = omega lo z; inv32 = (1/m, 1/I), read only. */
    float* pos32lo;
    float* lo32;        /* float[n][4] */
    float* wlz32;       /* float[n] */
    float* inv32;       /* float[n][2] */
} tmps_atoms;

/* Full neighbor list with its contact history. */
typedef struct tmps_nlist {
    int32_t n;
    int32_t slots;
    int32_t* nbr;
    int32_t* nnb;
    uint64_t* touch;
    double* shear;
    double* rolling;         /* [3][slots][n] rolling displacement, or NULL (no rolling model) */
} tmps_nlist;

/* Contact law.  style: 0 gran/hooke, 1 gran/hooke/history, 2 gran/hertz,
 * 3 gran/hertz/history, 4 granular.  Model ids for granular follow
 * src/taichimps/GRANULAR/granular.py:50-64. */
typedef struct tmps_pair_params {
    int32_t style;
    int32_t normal_id;
    int32_t damping_id;
    int32_t tangential_id;
    int32_t limit_damping;
    int32_t pad_;
    double kn, kt, gamman, gammat, xmu;
    double damp, xt, mu;
    /* rolling resistance of pair granular (GRANULAR/rolling.py:16-50): 0 none, 1 epsd */
    int32_t rolling_id;
    int32_t pad2_;
    double k_roll, gamma_roll, mu_roll;
} tmps_pair_params;

/* Pressure servo / strain control for x, y, z (orthogonal box).
 * Styles: 0 none, 1 erate, 2 trate, 3 vel, 4 wiggle, 5 final, 6 delta,
 * 7 scale, 8 pressure, 9 pressure/mean, 10 volume (deform_pressure.py:76-82).
 * The volume style and the box style (isotropic volume or mean-pressure
 * control of the whole box) run after the per-axis updates, in one thread,
 * when `post` is set (deform_pressure.py:858-1001). */
typedef struct tmps_servo {
    int32_t style[3];
    int32_t couple;     /* 0 none, 1 xyz, 2 xy, 3 yz, 4 xz */
    int32_t normalize;
    int32_t remap;      /* 0 none, 1 x, 2 v */
    double max_rate;
    double rate[3], vel[3], scale[3], flo[3], fhi[3], dlo[3], dhi[3];
    double amp[3], tper[3], ptarget[3], pgain[3];
    double lo_start[3], hi_start[3];
    double cum[3];      /* cumulative shift of pressure-controlled axes */
    double pressure[6]; /* last pressure tensor servoed on (output) */
    /* counters used by the fused step (deform_pressure.py:1121-1123): */
    int64_t nsteps;       /* updates since setup: elapsed = nsteps * dt */
    int64_t nsteps_total; /* run length for final/delta/scale */
    int64_t step_count;   /* end_of_step calls, for nevery */
    int32_t nevery;
    int32_t post;         /* volume or box styles present: run the post-pass */
    /* volume style links (_setup_volume_links, deform_pressure.py:358-380):
     * vsub 0 one_from_one, 1 one_from_two, 2 two_from_one */
    int32_t vsub[3], vfixed[3], vdyn1[3], vdyn2[3];
    int32_t vol_balance_p;
    int32_t box_style;    /* 0 none, 1 volume, 2 pressure (set_box) */
    double vol_start;     /* box volume at setup */
    double box_ptarget, box_pgain;
    double box_vshift[3]; /* cumulative_vshift of the box pressure style */
    /* last step's strain rate and pressure per axis (vol/balance/p) */
    double prior_rate[3], prior_pressure[3];
    int32_t saved;        /* prior_* hold a step */
    int32_t pad2_;
} tmps_servo;

/* State of the fused step (tmps_fused_*), device-resident.  One step of
 * Simulation._sub_step_inner (simulation.py:205-247) with fix nve/sphere,
 * optional damping/cundall and optional deform/pressure is three launches:
 *   A  second half-kick of the previous step + pending remap x + first
 *      half-kick + drift + skin check
 *   C  contact forces + Cundall damping + the virial (pair + kinetic) as
 *      per-block partial sums
 *   S  (with deform/pressure) virial total -> pressure -> servo -> new box
 * A step whose skin check asks for a rebuild sets `aborted` in C; every
 * later fused launch then returns at once, so many steps can be queued (or
 * replayed as a CUDA graph) and the host rebuilds only when one does. */
typedef struct tmps_engine {
    int64_t step;            /* timestep of the last completed step */
    int64_t last_build_step; /* timestep of the last neighbor build */
    int32_t aborted;         /* a step needs a rebuild: later fused launches do nothing */
    int32_t disp_stamp;      /* set to the step number when an atom moved more than skin/2 */
    int32_t final_pending;   /* v holds v(t+dt/2): the last force's second half-kick is pending */
    int32_t delay, every, check; /* neigh_modify (neighbor.py:88-95) */
    int32_t cundall;         /* apply damping/cundall in C */
    int32_t servo;           /* a deform/pressure fix is present */
    int32_t mixed;           /* 1: split FP64 positions + FP32 contact arithmetic */
    int32_t single_bin[3];   /* periodic dimension with one bin (FP32 image in C) */
    int32_t nblocks;         /* virial partials: blocks of A + blocks of C */
    double dt, gamma_lin, gamma_ang, trigger_sq;
    double lo0[3], h0[3];    /* box origin and bin size at the last build (mixed) */
    float dlo32[4], dh32[4]; /* lo - lo0, h - h0 (mixed skin check) */
    float h32[4], prd32[4], iprd32[4];
    float hlo32[4], prdlo32[4]; /* low words: h = h32 + hlo32, prd = prd32 + prdlo32 */
    double remap_scale[3];   /* new prd / old prd of the pending remap */
    double pad2_;
    /* FP32 copies of per-step constants, so no thread converts a double */
    float dt_hi, dt_lo, trigger32, gamma_lin32, gamma_ang32, pad3_;
    float eps_hi[4], eps_lo[4]; /* remap_scale - 1 as a double word (mixed) */
    /* Exact culling of contact-free atom groups in C's first pass (set by
     * tmps_fused_bounds): a group whose smallest gap at the reference
     * positions exceeds 2 sqrt(maxd2) + shift_bound + cull_tol holds no
     * contact. */
    double prd_ref[3];       /* box lengths at the reference */
    int64_t part_off;        /* byte offset of the virial partials in the scratch */
    float shift_bound;       /* running max of sum_d |prd_d - prd_ref_d| */
    uint32_t maxd2_bits;     /* running max of |x - x0|^2 over atoms and steps, FP32 bits */
    int32_t cull;            /* 1: the per-group gaps in the scratch are valid */
    float cull_tol;          /* absolute slack for the FP32 rounding of the test */
    /* Optional per-step record of the servo's pressure tensor in host memory
     * (tmps_fused_pressure_log): step s writes plog[(s % plog_len) * 6 + k]. */
    double* plog;            /* device address of a pinned host array, or NULL */
    int32_t plog_len;
    int32_t order_ready;     /* 1: C walks the groups in the ascending gap order
                              * tmps_fused_bounds left in the scratch (set by S
                              * after the first step that follows the bounds) */
    int64_t stop_step;       /* fused launches do nothing once step >= stop_step (batched runs) */
    int32_t touching;        /* atoms whose gap bound at the last tmps_fused_bounds is <= 0 */
    int32_t kick_all;        /* set by tmps_fused_prepare when some 1/m or 1/I is not a positive
                              * finite number (or dt <= 0): the FP64 update then kicks every atom;
                              * else it skips the kick of an atom whose force and torque are exact
                              * zeros (its C flag clear), which would leave it unchanged */
} tmps_engine;

/* One instance of a batched run (tmps_batch_*): the device state of one
 * independent system -- its own atoms, list, pair coefficients, box, servo,
 * fused-step engine and scratch, exactly what the single-instance calls take --
 * and the range of blocks it owns in each batched grid.  Its grids are the
 * ones a single-instance launch of the same launch shape uses
 * (tmps_fused_shape), so a batched step and a single-instance step of the
 * same instance and shape are interchangeable. */
typedef struct tmps_instance {
    tmps_atoms a;
    tmps_nlist nl;
    tmps_pair_params p;
    tmps_box* box;
    tmps_engine* eng;
    tmps_servo* servo;
    void* scratch;           /* tmps_fused_scratch_bytes(n, style, mixed) bytes */
    int32_t a_first, a_blocks; /* blocks [a_first, a_first + a_blocks) of the batched A grid */
    int32_t c_first, c_blocks; /* ... of the batched C grid */
} tmps_instance;

/* ---- library ---------------------------------------------------------- */

/* Version and build identity; no reference counterpart. */
const char* tmps_version(void);

/* Kernels launched by this library since it was loaded (all entry points);
 * no reference counterpart. */
long long tmps_launch_count(void);

/* The CUDA runtime's last error on this host thread, by name and text
 * (left set; an entry point that returned TMPS_ERR_CUDA left it there);
 * no reference counterpart. */
const char* tmps_last_cuda_error(void);

/* Copies a host box into device memory (Domain._sync, domain.py:235-254). */
int tmps_box_set(tmps_box* d_box, const tmps_box* h_box, void* stream);

/* ---- integrator / fixes ----------------------------------------------- */

/* FixNVESphere.initial_integrate (src/taichimps/EXTRA_FIX/nve_sphere.py:44-77,155-162). */
int tmps_verlet_initial(const tmps_atoms* a, double dt, void* stream);

/* FixNVESphere.final_integrate (src/taichimps/EXTRA_FIX/nve_sphere.py:79-96,164-171). */
int tmps_verlet_final(const tmps_atoms* a, double dt, void* stream);

/* AtomSystem.clear_forces (src/taichimps/atom.py:201-220). */
int tmps_clear_forces(const tmps_atoms* a, void* stream);

/* ---- particle input and output ---------------------------------------- */

/* AtomSystem.add_particles (src/taichimps/atom.py:55-145) for a system's first
 * n = a->n particles: writes xr, vm, om (rmass = (4/3) pi r^3 density, moment
 * of inertia 0.4 m r r), tag (1..n when `tag` is NULL), uid = 0..n-1, and
 * zeroes f, torque, x0 and virial.  x, v, omega: double[n][3] (v, omega NULL:
 * zero); radius, density: double[n], or NULL for radius_value /
 * density_value on every atom.  Each input may be device memory or
 * page-locked host memory (read in place); pageable memory is refused
 * (TMPS_ERR_BAD_ARG).  *d_max_radius (device double) receives the largest
 * radius. */
int tmps_atoms_assemble(const tmps_atoms* a, const double* x, const double* v, const double* omega,
                        const double* radius, double radius_value, const double* density, double density_value,
                        const int32_t* tag, double* d_max_radius, void* stream);

/* Fields of tmps_atoms_read (the Taichi fields of src/taichimps/atom.py:36-55). */
enum {
    TMPS_FIELD_X = 0,       /* double[n][3] */
    TMPS_FIELD_V = 1,       /* double[n][3] */
    TMPS_FIELD_OMEGA = 2,   /* double[n][3] */
    TMPS_FIELD_RADIUS = 3,  /* double[n] */
    TMPS_FIELD_RMASS = 4,   /* double[n] */
    TMPS_FIELD_F = 5,       /* double[n][3] */
    TMPS_FIELD_TORQUE = 6,  /* double[n][3] */
    TMPS_FIELD_VIRIAL = 7,  /* double[n][6] */
};

/* The field's to_numpy(): its rows in insertion order (row j = the atom with
 * uid j) into `out`, device memory or page-locked host memory (written in
 * place).  d_slot_of: int32[n] device scratch. */
int tmps_atoms_read(const tmps_atoms* a, int32_t field, int32_t* d_slot_of, double* out, void* stream);

/* FixDampingCundall.post_force (src/taichimps/EXTRA_FIX/damping_cundall.py:36-63). */
int tmps_damping_cundall(const tmps_atoms* a, double gamma_lin, double gamma_ang, void* stream);

/* NeighborList.check_displacement (src/taichimps/neighbor.py:214-245).
 * Sets *d_flag (device int32) to `stamp` when some atom moved more than
 * half the skin since the last build. */
int tmps_skin_check(const tmps_atoms* a, double trigger_sq, int32_t stamp, int32_t* d_flag,
                    void* stream);

/* Domain.pbc (src/taichimps/domain.py:560-584): wrap, plus the remap-v kick. */
int tmps_pbc(const tmps_atoms* a, const tmps_box* d_box, void* stream);

/* ---- neighbor list and contact history -------------------------------- */

/* Scratch size (bytes) tmps_nlist_build needs for n atoms and ncell cells. */
int64_t tmps_nlist_workspace_bytes(int32_t n, int32_t ncell);

/* NeighborList.build (src/taichimps/neighbor.py:247-369,414-435): bins atoms
 * by cell in lamda coordinates (grid g/csize already in d_box, `ncell` =
 * gx*gy*gz), sorts them by cell (cells in Morton order, insertion order
 * within a cell), permutes every per-atom array from `src` into `dst`, and
 * builds the full list into `nl` (cut (ri + rj + skin)^2, exact FP64).
 * `order` (int32[n]) receives, for each new slot, the old internal index;
 * `cell_rank` (int32[ncell]) is the Morton rank of each linear cell id;
 * `cell_of` (int32[n]) receives each atom's linear cell id in the new order.
 * Row overflow sets TMPS_STATUS_NLIST_OVERFLOW in *d_status. */
int tmps_nlist_build(const tmps_atoms* src, const tmps_atoms* dst, const tmps_box* d_box,
                     int32_t ncell, double skin, const int32_t* cell_rank, int32_t* order,
                     int32_t* cell_of, const tmps_nlist* nl, void* workspace,
                     int64_t workspace_bytes, int32_t* d_status, void* stream);

/* No counterpart in the reference: tmps_nlist_build for callers that cannot
 * allocate device memory at all -- a host whose device memory all belongs to
 * its own fixed arena, a host whose step loop must not enter the CUDA
 * allocator (an allocation can synchronise the device and stall the loop),
 * or a foreign-language host that can only pass the arrays it registered.
 * Same arguments and results as tmps_nlist_build minus the workspace: the
 * scratch is one static device array built into the library (about 23 MB,
 * held by every GPU that loads the library until the process exits), so it
 * takes at most TMPS_NOALLOC_MAX_ATOMS atoms and TMPS_NOALLOC_MAX_CELLS grid
 * cells (the reference's own cell cap) and returns TMPS_ERR_TOO_LARGE beyond
 * that.  It calls no allocator.  It runs the kernels of tmps_nlist_build,
 * the FP32 pre-test of the candidate pairs included (its cell-local offsets
 * take 16 MB of the array): the same pair set at the same speed.  The first
 * call on a device looks up the scratch's device address
 * (cudaGetSymbolAddress) and keeps it for the life of the process, so make
 * that first call before any stream capture, and do not use the library
 * across a cudaDeviceReset (the kept address belongs to the old context).
 * Every call shares the one scratch (the counters are cleared at the start of
 * each call): calls whose work overlaps on the GPU -- other streams, other
 * host threads -- race; order them on one stream. */
int tmps_nlist_build_noalloc(const tmps_atoms* src, const tmps_atoms* dst, const tmps_box* d_box,
                             int32_t ncell, double skin, const int32_t* cell_rank, int32_t* order,
                             int32_t* cell_of, const tmps_nlist* nl, int32_t* d_status, void* stream);

/* ContactHistory.save_state + restore_state (src/taichimps/contact_history.py:91-153):
 * carries every touching contact of the old list onto the new list, keyed by
 * the partner's identity, zeroing the rest.  `order` maps new -> old index. */
int tmps_history_remap(const tmps_nlist* old_nl, const tmps_nlist* new_nl, const int32_t* order,
                       void* stream);

/* ---- contact force ------------------------------------------------------ */

/* GranularPair.compute for every style (src/taichimps/GRANULAR/base.py:25-38,
 * hooke.py:52-173, hooke_history.py:71-217, hertz.py:46-148,
 * hertz_history.py:57-193, granular.py:282-452): full list, one thread per
 * atom, no atomics; each contact is evaluated in one fixed orientation
 * (lower internal index first) by both of its atoms, so the two copies of
 * its shear stay exact negatives.  accumulate != 0 adds into
 * f/torque/virial (the reference's atomic_add semantics); 0 overwrites
 * them (clear_forces fused in). */
int tmps_contact(const tmps_atoms* a, const tmps_nlist* nl, const tmps_box* d_box,
                 const tmps_pair_params* p, double dt, int32_t shearupdate, int32_t accumulate,
                 void* stream);

/* ComputeContactAtom.compute (src/taichimps/computes/contact_atom.py:21-63):
 * per atom (internal order) into d_count (device int32[n]) the number of
 * neighbors with rsq < (ri + rj)^2 and rsq > 1e-18, each contact counted for
 * both partners (the coordination number). */
int tmps_contact_count(const tmps_atoms* a, const tmps_nlist* nl, const tmps_box* d_box, int32_t* d_count,
                       void* stream);

/* ---- virial, pressure servo, remap ------------------------------------- */

/* Computes.compute_virial_kernel (src/taichimps/computes/thermo.py:62-109):
 * sum of the per-atom virial (+ sum m v_a v_b when keflag) into d_out[6]
 * (device), deterministic order. */
int tmps_virial_reduce(const tmps_atoms* a, int32_t keflag, double* d_out, void* workspace,
                       int64_t workspace_bytes, void* stream);

/* Scratch size (bytes) tmps_virial_reduce needs for n atoms. */
int64_t tmps_virial_workspace_bytes(int32_t n);

/* FixDeformPressure._servo_kernel (src/taichimps/EXTRA_FIX/deform_pressure.py:598-702)
 * with the host path's styles for x/y/z: pressure from d_virial / volume,
 * couple, normalize, max/rate, new box into d_box (old box kept in
 * d_box->old_lo/old_prd and remap_pending set for remap x). */
int tmps_servo_step(tmps_box* d_box, tmps_servo* d_servo, const double* d_virial, double elapsed,
                    double frac, double dt, int32_t* d_status, void* stream);

/* ---- fused step ---------------------------------------------------------
 * The mixed form keeps positions split: an FP64 offset from the origin of
 * the atom's cell at the last build (xr.xyz holds the offset, cell32 the
 * cell as cx | cy << 10 | cz << 20), so an affine remap is a scale of the
 * offset and the FP32 copies the contact kernel reads are exact to 1e-7 of a
 * bin, not of the box.  pos32 = (offset, r), vel32 = (v, m), om32 = (w, I). */

/* After a neighbor build: 1/m and 1/I for the fused step and, with
 * d_eng->mixed, the split positions (offset from each atom's cell origin in
 * xr, cell32, FP32 copies, o0_32) and FP32 copies of f and torque into f32,
 * torque32.  `cell_of` is the linear cell id from tmps_nlist_build; records
 * lo0 / h0 in d_eng, clears d_eng->touching for tmps_fused_bounds and sets
 * d_eng->kick_all. */
int tmps_fused_prepare(const tmps_atoms* a, const tmps_box* d_box, tmps_engine* d_eng,
                       const int32_t* cell_of, void* stream);

/* The per-contact histories (shear, rolling) of the touching slots between
 * their two storages: to_dw 1 turns each double into an FP32 double word
 * (hi, lo) in the same 8 bytes -- the mixed form's contact pass reads and
 * writes them that way -- and to_dw 0 turns them back into doubles (exact for
 * values of at most 48 significant bits).  Call with 1 after
 * tmps_fused_prepare of a mixed run, with 0 before the history is carried
 * across a rebuild, saved or read, and at the end of the run. */
int tmps_mixed_history(const tmps_nlist* nl, int32_t to_dw, void* stream);

/* Back from the mixed form to absolute FP64 positions in xr, and the FP32
 * force and torque into f / torque. */
int tmps_mixed_unpack(const tmps_atoms* a, const tmps_box* d_box, void* stream);

/* After tmps_fused_prepare, with the list of the last build: per 32-atom
 * group, the smallest gap |d| - (ri + rj) at the build positions x0 (into
 * `scratch`), and every flag word set.  Resets the running bounds in d_eng;
 * cull = 0 leaves culling off (C then screens every group).  No reference
 * counterpart: it lets C skip groups that cannot touch without changing any
 * result. */
int tmps_fused_bounds(const tmps_atoms* a, const tmps_nlist* nl, const tmps_box* d_box, tmps_engine* d_eng,
                      const tmps_pair_params* p, int32_t cull, void* scratch, void* stream);

/* Launch A (see tmps_engine).  `scratch` is C's: A reads the flag words of
 * the last C (an unflagged atom's force and torque are exact zeros and are
 * not loaded) and writes the first virial partials, the kinetic term
 * sum m v v of every atom at mid-step velocity.  a_blocks: A's grid from
 * tmps_fused_shape, or <= 0 for the default. */
int tmps_fused_a(const tmps_atoms* a, tmps_box* d_box, tmps_engine* d_eng, int32_t a_blocks, void* scratch,
                 void* stream);

/* Launch C: per 32-atom group a bound check (tmps_fused_bounds), a screen of
 * the atoms the bounds leave (finishes contact-free ones, flags the rest) and
 * the contact law over the flagged ones.  `scratch` (tmps_fused_scratch_bytes(n),
 * caller memory: flag words, per-group and per-atom gaps, then the
 * d_eng->nblocks virial partial sums, A's blocks then C's).  c_blocks: C's
 * grid from tmps_fused_shape, or <= 0 for the default; d_eng->nblocks must be
 * A's blocks + C's blocks of the same shape.  rows != 0 takes the per-atom-row
 * path instead: every atom's row, one thread per atom, no group ruled out --
 * for contact-dense states, where the screen rules out almost nothing.  Both
 * paths sum each atom's contacts in slot order and keep the flag words'
 * meaning, so they may alternate between builds. */
int tmps_fused_c(const tmps_atoms* a, const tmps_nlist* nl, const tmps_box* d_box, tmps_engine* d_eng,
                 const tmps_pair_params* p, int32_t c_blocks, void* scratch, int32_t rows, void* stream);

/* Launch S: rebuild decision, virial total (from C's scratch), servo. */
int tmps_fused_servo(tmps_box* d_box, tmps_servo* d_servo, tmps_engine* d_eng, const void* scratch,
                     int32_t* d_status, void* stream);

/* Number of virial partial sums A and C write for n atoms with this pair
 * style (tmps_pair_params.style) in this form (mixed 0/1) under the default
 * launch shape: one per block of A and of C, at most one resident wave each. */
int32_t tmps_fused_blocks(int32_t n, int32_t style, int32_t mixed);

/* Launch shape: the grids of A and C for n atoms when each warp takes
 * a_groups_per_warp (A) or c_groups_per_warp (C) 32-atom groups: one block of
 * A per 256 x a_groups_per_warp atoms, one block of C per 128 x
 * c_groups_per_warp atoms, never more than the default grid (<= 0: the
 * default, the grids tmps_fused_blocks counts).  No reference counterpart
 * (launch geometry).  The virial is summed per block, so the shape fixes the
 * summation order: results depend on it at rounding level only, and two runs
 * with the same shape are bit-identical. */
int tmps_fused_shape(int32_t n, int32_t style, int32_t mixed, int32_t a_groups_per_warp, int32_t c_groups_per_warp,
                     int32_t* a_blocks, int32_t* c_blocks);

/* Scratch bytes tmps_fused_c / tmps_fused_servo need (same arguments). */
int64_t tmps_fused_scratch_bytes(int32_t n, int32_t style, int32_t mixed);

/* Records the servo's pressure tensor of every fused step into h_log, pinned
 * (page-locked, device-mapped) host memory of len x 6 doubles: step s writes
 * row s % len, from the device, with no host synchronisation.  h_log = NULL
 * stops recording.  The reference's host servo path reads this tensor back
 * every step (deform_pressure.py:1113-1219); this is that read without the
 * round trip. */
int tmps_fused_pressure_log(tmps_engine* d_eng, double* h_log, int32_t len, void* stream);

/* FP64 pipe probe (no reference counterpart; the FP64 form's roofline
 * denominator): eight independent DFMA chains of `iters` steps per thread on
 * a grid of blocks x threads (threads a multiple of 32, at most 256); time it
 * on `stream` and count 8 x iters x blocks x threads DFMA.  Each thread
 * writes one double to d_out (blocks x threads slots); nothing is allocated. */
int tmps_probe_fp64(int32_t blocks, int32_t threads, int32_t iters, double* d_out, void* stream);

/* Self-check of the library's integer-operation double<->float conversions
 * against the hardware's rounding: which 0 (float)a, 1 (double)(float)a,
 * 2 the hi + lo split of a (two outputs per operand).  d_mine and d_hw
 * (n doubles, 2n for which 2) must agree bit for bit.  No reference
 * counterpart. */
int tmps_selftest_arith(int32_t which, const double* d_a, int32_t n, double* d_mine, double* d_hw, void* stream);

/* ---- batched runs ----------------------------------------------------------
 * Many independent systems of uneven size (each with its own box, contact
 * coefficients and servo) advance together: one launch of each of A, C and S
 * per step covers every instance.  No reference counterpart (the reference
 * runs one system per process); each instance's arithmetic is the
 * single-instance fused step's.  d_inst is a device array of ninst
 * tmps_instance; d_block_inst maps every block of the A (or C) grid to its
 * instance.  All instances share the arithmetic form (mixed) and the pair
 * style. */

/* Blocks one instance of n atoms owns in the A and C grids under the default
 * launch shape (tmps_fused_shape with both counts 0).  An instance may
 * own any grid tmps_fused_shape gives; its engine's nblocks must match. */
int tmps_batch_blocks(int32_t n, int32_t style, int32_t mixed, int32_t* a_blocks, int32_t* c_blocks);

int tmps_batch_a(const tmps_instance* d_inst, const int32_t* d_block_inst, int32_t nblocks, int32_t mixed,
                 void* stream);
int tmps_batch_c(const tmps_instance* d_inst, const int32_t* d_block_inst, int32_t nblocks, int32_t style,
                 int32_t mixed, void* stream);
/* S for every instance, one block each; a box driven non-positive sets
 * TMPS_STATUS_BOX_NONPOSITIVE in *d_status. */
int tmps_batch_servo(const tmps_instance* d_inst, int32_t ninst, int32_t* d_status, void* stream);
/* d_state[2 i] = step, d_state[2 i + 1] = aborted of instance i (one copy for the host). */
int tmps_batch_state(const tmps_instance* d_inst, int32_t ninst, int64_t* d_state, void* stream);

/* Applies what the fused step leaves pending -- the second half-kick of the
 * last step and a remap x the servo asked for -- so the state is that of the
 * reference at the end of a step. */
int tmps_fused_settle(const tmps_atoms* a, tmps_box* d_box, tmps_engine* d_eng, void* stream);

/* FixDeformPressure.remap_positions (src/taichimps/EXTRA_FIX/deform_pressure.py:493-530):
 * x from the old box's lamda coordinates into the new box; clears
 * remap_pending. */
int tmps_remap_x(const tmps_atoms* a, tmps_box* d_box, void* stream);

/* ---- granular walls ------------------------------------------------------
 * The wall is a contact partner of zero radius and infinite mass: radsum =
 * Reff = r_i, meff = m_i, moment arm the full radius.  One history slot per
 * atom, indexed by the atom's insertion index (tmps_atoms.uid) so it follows
 * the atom through the neighbor build's re-sort. */
typedef struct tmps_wall_params {
    int32_t kind;            /* 0 plane (FixWallGran), 1 cylinder side (FixWallGranRegion) */
    int32_t axis;            /* plane: normal axis; cylinder: cylinder axis (0, 1, 2) */
    int32_t side;            /* plane: -1 wall below the atoms (normal +axis), +1 above;
                                cylinder: -1 atoms inside, +1 outside */
    int32_t history;         /* keep the shear history (the .../history styles) */
    int32_t hertz;           /* cylinder: hertz normal, forces scaled by sqrt(r_i delta) */
    int32_t limit_damping;
    int32_t shear_axis;      /* plane: axis of the in-plane wall velocity, or -1 */
    int32_t has_axis_bounds; /* cylinder: only atoms with axis_lo <= x_axis <= axis_hi */
    double coord;            /* plane: wall position this step */
    double vwall_n;          /* plane: wall velocity along its normal axis this step (wiggle) */
    double vwall_s;          /* plane: in-plane wall velocity (shear) */
    double c1, c2, radius;   /* cylinder: centre in the cross-section, radius */
    double axis_lo, axis_hi;
    double kn, kt, gamman, gammat, xmu;
} tmps_wall_params;

/* FixWallGran.post_force_kernel (EXTRA_FIX/wall_gran.py:143-228) for kind 0,
 * FixWallGranRegion.post_force_kernel (EXTRA_FIX/wall_gran_region.py:134-276)
 * for kind 1: adds the wall force and torque to f / torque.  d_shear
 * double[3][nslots], d_touch int32[nslots] (nslots > every uid). */
int tmps_wall_gran(const tmps_atoms* a, const tmps_wall_params* p, double dt, int32_t history_update,
                   double* d_shear, int32_t* d_touch, int32_t nslots, void* stream);

/* ---- differentiable run (hand-written adjoint) --------------------------
 * gran/hertz/history (GRANULAR/hertz_history.py:57-171) + fix nve/sphere
 * (EXTRA_FIX/nve_sphere.py:43-96) + fix deform/pressure with x/y/z styles
 * none, erate and pressure, couple and max/rate, remap x
 * (EXTRA_FIX/deform_pressure.py:493-530, 583-702), in FP64 on a fully
 * periodic orthogonal box.  Atoms stay in the caller's order (never
 * re-sorted); contacts are a half pair list (i < j) sorted by (i, j) with
 * the history in the i -> j sense.  Per-atom sums gather over the pairs in a
 * fixed order (no atomics), so a run is bit-reproducible.  The adjoint of a
 * step replays the forward's recorded masks (contact on, Coulomb slip,
 * |shear| != 0, damping clamp; the servo's max/rate clamp): no smoothing.
 * All arrays are device memory owned by the caller; [3][n] is
 * component-major. */

typedef struct tmps_adj_params {
    double kn, kt, gamman, gammat, xmu;
    double dt;
    int32_t limit_damping;
    int32_t pad_;
} tmps_adj_params;

typedef struct tmps_adj_servo {
    int32_t style[3];    /* 0 none, 1 erate, 8 pressure (the codes of tmps_servo) */
    int32_t couple;      /* 0 none, 1 xyz, 2 xy, 3 yz, 4 xz */
    int32_t normalize;   /* normalize/pressure */
    int32_t pad_;
    double rate[3], ptarget[3], pgain[3];
    double lo_start[3], hi_start[3];
    double max_rate;
} tmps_adj_servo;

/* Box after a step (record s; record 0 is the box at setup), device. */
typedef struct tmps_adj_rec {
    double lo[3], prd[3], cum[3];
    double w[6];         /* virial (pair + kinetic) total of step s, [xx, yy, zz, xy, xz, yz] */
    double q;            /* deviatoric stress p_zz - (p_xx + p_yy) / 2 of step s */
    double elapsed;      /* servo time of step s */
    int32_t clamp;       /* bit d: axis d's servo rate hit max/rate */
    int32_t pad_;
} tmps_adj_rec;

typedef struct tmps_adj_sys {
    int32_t n;
    int32_t npairs;
    double* x;           /* [3][n] state at the end of the last step */
    double* v;
    double* w;
    double* f;           /* forces and torques of the last step */
    double* t;
    const double* radius;   /* [n] */
    const double* mass;     /* [n] */
    double* shear;          /* [3][npairs] */
    const int32_t* pi;      /* [npairs] */
    const int32_t* pj;      /* [npairs] */
    const int32_t* ibeg;    /* [n + 1]: pairs with pi == a are ibeg[a] .. ibeg[a + 1] - 1 */
    const int32_t* jbeg;    /* [n + 1]: jlist[jbeg[a] .. jbeg[a + 1] - 1] are the pairs with pj == a */
    const int32_t* jlist;   /* [npairs] */
} tmps_adj_sys;

/* One step's record for the reverse pass. */
typedef struct tmps_adj_tape {
    double* xh;          /* [3][n] after the first half-kick and the drift */
    double* vh;
    double* wh;
    double* f;           /* [3][n] forces and torques the step computed */
    double* t;
    double* shear;       /* [3][npairs] history entering the contact pass */
    uint8_t* mask;       /* [npairs] */
} tmps_adj_tape;

/* Adjoint state, carried backwards step by step. */
typedef struct tmps_adj_bar {
    double* x;           /* [3][n] */
    double* v;
    double* w;
    double* f;
    double* t;
    double* shear;       /* [3][npairs] */
    double* radius;      /* [n] dL/dr through radius directly (mass terms are in `mass`) */
    double* mass;        /* [n] dL/dm */
    double* params;      /* [8]: dL/d kn, kt, gamman, gammat, xmu */
    double* box;         /* [2][9]: (lo, prd, cum) adjoints of the boxes of records n and n + 1, by parity */
} tmps_adj_bar;

/* Workspace for the adjoint-run calls (bytes). */
int64_t tmps_adj_workspace_bytes(int32_t n, int32_t npairs);

/* Pair list build (NeighborList.build_neighbor_list, neighbor.py:305-369, as
 * a half list in the caller's order): pairs i < j with |d|^2 < (ri + rj +
 * skin)^2 under the minimum image.  First call with d_pj = NULL fills
 * d_count[i]; the second, with d_ibeg = exclusive prefix of the counts, fills
 * d_pi / d_pj in (i, j) order. */
int tmps_adj_pairs(int32_t n, const double* d_x, const double* d_radius, const tmps_adj_rec* d_box, double skin,
                   int32_t* d_count, const int32_t* d_ibeg, int32_t* d_pi, int32_t* d_pj, void* stream);

/* For each old pair, its index in a new list (-1 if gone); the history
 * carried across a rebuild (contact_history.py:91-139 keyed by the pair). */
int tmps_adj_pair_map(int32_t nold, const int32_t* d_old_pi, const int32_t* d_old_pj, const int32_t* d_new_ibeg,
                      const int32_t* d_new_pj, int32_t* d_map, void* stream);
/* reverse = 0: new[map[p]] = old[p] (new zeroed first); 1: old[p] = new[map[p]] or 0. */
int tmps_adj_carry(int32_t nold, int32_t nnew, const int32_t* d_map, double* d_old, double* d_new, int32_t reverse,
                   void* stream);

/* Setup force evaluation (Simulation.setup: pair compute with shearupdate
 * off) on the state: f, t and the history; `tape` records the history and
 * the masks. */
int tmps_adj_setup(const tmps_adj_sys* s, const tmps_adj_params* p, const tmps_adj_rec* d_box,
                   const tmps_adj_tape* tape, void* work, void* stream);

/* First half of step s: half-kick and drift into tape->xh/vh/wh; the
 * largest |xh - d_xbuild|^2 goes to *d_disp (as FP64 bits, for the host's
 * rebuild decision, neighbor.py:214-245). */
int tmps_adj_initial(const tmps_adj_sys* s, const tmps_adj_params* p, const tmps_adj_tape* tape,
                     const double* d_xbuild, uint64_t* d_disp, void* stream);

/* Rest of step s: contacts (shearupdate on), second half-kick, pressure,
 * servo and remap; writes d_rec[s] from d_rec[s - 1]. */
int tmps_adj_finish(const tmps_adj_sys* s, const tmps_adj_params* p, const tmps_adj_servo* sv,
                    const tmps_adj_tape* tape, tmps_adj_rec* d_rec, int64_t step, void* work, void* stream);

/* Reverse of step s (from d_rec[s - 1] to d_rec[s]), given the adjoint of
 * the state after it in `b`; leaves the adjoint of the state before it.
 * `qbar` is dL/dq of step s; d_fprev / d_tprev the forces step s started
 * from. */
int tmps_adj_step_back(const tmps_adj_sys* s, const tmps_adj_params* p, const tmps_adj_servo* sv,
                       const tmps_adj_tape* tape, const tmps_adj_rec* d_rec, int64_t step, const double* d_fprev,
                       const double* d_tprev, double qbar, const tmps_adj_bar* b, void* work, void* stream);

/* Reverse of the setup force evaluation: adds its radius, mass and
 * parameter terms; `b->x`, `b->v`, `b->w` receive the adjoint of the
 * initial state. */
int tmps_adj_setup_back(const tmps_adj_sys* s, const tmps_adj_params* p, const tmps_adj_rec* d_box,
                        const tmps_adj_tape* tape, const tmps_adj_bar* b, void* work, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TAICHIMPS_GB300_H */
