/*
 * demsph_gb300.h - C ABI of the GB300-native coupled DEM-SPH step.
 *
 * The reference (kaiqideng/DEM-SPHSource) has no plugin or FFI interface: its
 * engine boundary is five C++ host functions that take the device data by
 * reference,
 *     neighborSearch                       core/neighborSearch.h:28
 *     solidIntegrateBeforeContact          core/integrate.h:43
 *     fluidIntegrate                       core/integrate.h:19
 *     calSolidContactAfterFluidIntegrate   core/integrate.h:41
 *     solidIntegrateAfterContact           core/integrate.h:45
 * plus the DeviceData life cycle (copy / uploadState / release,
 * core/deviceStructs.h) driven by class dataBase (core/dataBase.cpp:192-260,
 * 434-449).  This header replaces exactly that boundary with plain C: an
 * opaque engine handle, host pointers and sizes, and a status code on every
 * call.  Nothing here aborts; device memory is owned by the engine.
 *
 * Conventions
 *   - double3 data is passed as 3 interleaved doubles per element (the memory
 *     layout of std::vector<double3>), quaternions as 4 and symmetric
 *     matrices as 6 (xx, yy, zz, xy, xz, yz) - the reference's host layouts.
 *   - Indices are the reference's: fluid and solid particles numbered in the
 *     order they were added (core/hostStructs.h).
 *   - Output pointers may be NULL to skip a field.
 *   - Calls on one engine are not thread-safe; different engines are
 *     independent.  Work is issued on the engine's own CUDA stream; download
 *     and export calls synchronise that stream.
 *
 * The scene builder (demsph_builder_*) is the host-side mirror of the
 * reference's setup API (class dataBase, core/dataBase.h:33-219): the same
 * calls, argument meanings and validation, producing the arrays the engine
 * (and the FP64 oracle) take.
 */
#ifndef DEMSPH_GB300_H
#define DEMSPH_GB300_H

#include <stddef.h>

#if defined(__GNUC__)
#define DEMSPH_API __attribute__((visibility("default")))
#else
#define DEMSPH_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef enum demsph_status {
    DEMSPH_OK = 0,
    DEMSPH_ERR_ARGUMENT = 1,      /* bad pointer, index, size or parameter */
    DEMSPH_ERR_STATE = 2,         /* call out of order (e.g. a step before initialize) */
    DEMSPH_ERR_CUDA = 3,          /* a CUDA runtime call failed; see demsph_last_error */
    DEMSPH_ERR_NO_DEVICE = 4,     /* no usable CUDA device / wrong architecture */
    DEMSPH_ERR_CAPACITY = 5,      /* a neighbour or contact list overflowed; the engine grew it, re-run the step */
    DEMSPH_ERR_OUT_OF_MEMORY = 6,
    DEMSPH_ERR_TIMEOUT = 7,       /* a bounded device-side wait gave up */
    DEMSPH_ERR_IO = 8             /* a file could not be created or written */
} demsph_status;

/* Reference behaviours that can be switched off (all kept by default). */
enum {
    /* integrate.cu:540 returns from the wall loop at the first wall a particle
       does not touch, skipping later walls; the fix continues the loop. */
    DEMSPH_FIX_WALL_LOOP = 1,
    /* integrate.cu:919 reads clump orientations that are never integrated;
       the fix integrates the quaternion (FP64) each half step. */
    DEMSPH_FIX_CLUMP_ROTATION = 2
};

/* Everything class dataBase holds after the setup calls (HostData,
   core/hostStructs.h:387-398) plus the solver parameters, as host arrays. */
typedef struct demsph_scene {
    /* spatial grid and gravity (dataBase members, core/dataBase.h:243-246) */
    double domain_origin[3];
    double domain_size[3];
    double gravity[3];
    double time_step;
    int fluid_integrate_gap;
    double maximum_time;
    int num_frames;

    /* fluid particles (HostFluid, core/hostStructs.h:48-75) */
    int n_fluid;
    const double* fluid_position;        /* 3n */
    const double* fluid_velocity;        /* 3n */
    const double* fluid_acceleration;    /* 3n */
    const double* fluid_smoothing_length;/* n: points.effectiveRadii */
    const double* fluid_rho0;            /* n */
    const double* fluid_drho;            /* n */
    const double* fluid_sound_speed;     /* n */
    const double* fluid_nu;              /* n: kinematic viscosity */

    /* solid particles (HostSolid, core/hostStructs.h:77-117) */
    int n_solid;
    const double* solid_position;        /* 3n */
    const double* solid_velocity;        /* 3n */
    const double* solid_acceleration;    /* 3n */
    const double* solid_normal;          /* 3n */
    const double* solid_torque;          /* 3n */
    const double* solid_angular_velocity;/* 3n */
    const double* solid_effective_radius;/* n: points.effectiveRadii */
    const double* solid_radius;          /* n */
    const double* solid_inverse_mass;    /* n */
    const int* solid_material;           /* n */
    const int* solid_cluster;            /* n, -1 = none */
    const int* solid_clump;              /* n, -1 = none */
    const int* solid_is_dummy;           /* n, 1 = dummy wall particle */

    /* clumps (HostClump, core/hostStructs.h:119-152) */
    int n_clump;
    const double* clump_centroid;        /* 3n */
    const double* clump_velocity;        /* 3n */
    const double* clump_acceleration;    /* 3n */
    const double* clump_angular_velocity;/* 3n */
    const double* clump_torque;          /* 3n */
    const double* clump_orientation;     /* 4n: q0 q1 q2 q3 */
    const double* clump_inverse_inertia; /* 6n */
    const double* clump_inverse_mass;    /* n */
    const int* clump_pebble_start;       /* n */
    const int* clump_pebble_end;         /* n */

    /* infinite walls (HostInfiniteWall, core/hostStructs.h:154-174) */
    int n_wall;
    const double* wall_point;            /* 3n */
    const double* wall_normal;           /* 3n */
    const int* wall_material;            /* n */

    /* contact models per material pair (HostSolidContactModel,
       core/hostStructs.h:291-385); n_material*(n_material+1)/2 pair slots,
       slot index = getCombinedIndex (core/hostStructs.h:369-384) */
    int n_material;
    const double* hertzian;  /* 8 per slot: E G res k_r_k_s k_t_k_s mu_s mu_r mu_t */
    const double* linear;    /* 11 per slot: k_n k_s k_r k_t d_n d_s d_r d_t mu_s mu_r mu_t */
    const double* bonded;    /* 6 per slot: gamma E k_n_k_s sigma_s C mu */
} demsph_scene;

typedef struct demsph_options {
    int device;                  /* CUDA device ordinal (gpuPara.deviceIndex) */
    int fluid_neighbors_max;     /* fluid partners kept per fluid particle; 0 = 160 */
    int fluid_solids_max;        /* solid partners kept per fluid particle; 0 = 96 */
    int solid_contacts_per_particle; /* contact list capacity / solid count; 0 = 16 */
    int fixes;                   /* DEMSPH_FIX_* bits; 0 = reference behaviour */
    int debug;                   /* bit 0: keep each step's per-pair coupling forces for export */
    double solid_verlet_skin;    /* margin (m) of the solid contact candidates, rebuilt once a solid has
                                    moved half of it; 0 = 0.2 x the smallest solid radius; < 0 = no
                                    candidates: the reference's 27-cell walk every step */
    int fluid_lanes;             /* threads per fluid particle in the fluid list and pair loops (1, 2, 4
                                    or 8); 0 = chosen from the particle count */
    double fluid_verlet_skin;    /* margin (m) of the fluid list candidates, rebuilt (with the reorder of
                                    the fluids by cell) once a fluid or solid particle has moved half of
                                    it; 0 = 0.2 x the largest smoothing length; < 0 = no candidates: the
                                    reference's 27-cell walk every fluid step */
    int contact_rows_per_warp;   /* contact rows per warp of the solid contact-force kernel (4, 8, 16 or
                                    32); 0 = adapted to the contacts and bonds per row after every update.
                                    Results do not depend on it */
} demsph_options;

typedef struct demsph_counts {
    long long fluid_pairs;       /* fluid2Fluid.num: half list, i < j */
    long long fluid_solid_pairs; /* fluid2Solid.num */
    long long solid_pairs;       /* solid2Solid.num */
    long long bonds;             /* solidBond2Solid.num */
    long long bonds_intact;      /* bonds with isBonded == 1 */
    int grid_cells;              /* spatialGrid.num (cells + overflow bucket) */
    int grid_size[3];
    double cell_size[3];
} demsph_counts;

typedef struct demsph_engine demsph_engine;
typedef struct demsph_builder demsph_builder;

/* ---- status ---- */
DEMSPH_API const char* demsph_status_string(int status);
/* Last error message recorded on this engine ("" if none); valid until the next call. */
DEMSPH_API const char* demsph_last_error(const demsph_engine* e);
/* Library version string. */
DEMSPH_API const char* demsph_version(void);
/* Self-test of the bounded grid barrier the cooperative sorts use (no
   counterpart in the reference): two blocks of a cooperative launch wait at a
   barrier for 2 + missing arrivals, with a wait limit of a few milliseconds.
   With missing > 0 the wait runs out and the kernel records the timeout and
   returns (no fault, no hang); *status_out receives the device status bits:
   128 (barrier timeout) then, 0 when missing = 0.  Returns DEMSPH_OK when the
   launch itself ran. */
DEMSPH_API int demsph_selftest_barrier(int device, int missing, int* status_out);

/* ---- scene builder: the reference's setup API (core/dataBase.h:33-219) ---- */
/* HostSolidContactModel(n_material) as in solverBase::initialize (core/solverBase.cpp:16). */
DEMSPH_API demsph_builder* demsph_builder_new(int n_material);
DEMSPH_API void demsph_builder_free(demsph_builder* b);
DEMSPH_API const char* demsph_builder_last_error(const demsph_builder* b);
DEMSPH_API int demsph_builder_set_domain(demsph_builder* b, const double origin[3], const double size[3]); /* dataBase.h:93 */
DEMSPH_API int demsph_builder_set_gravity(demsph_builder* b, const double g[3]);                         /* dataBase.h:105 */
DEMSPH_API int demsph_builder_set_time_step(demsph_builder* b, double dt);                               /* dataBase.h:68 */
DEMSPH_API int demsph_builder_set_maximum_time(demsph_builder* b, double t);                             /* dataBase.h:38 */
DEMSPH_API int demsph_builder_set_num_frames(demsph_builder* b, int n);                                  /* dataBase.h:53 */
DEMSPH_API int demsph_builder_set_fluid_integrate_gap(demsph_builder* b, int gap);                       /* dataBase.h:83 */
DEMSPH_API int demsph_builder_set_hertzian(demsph_builder* b, int mi, int mj, double E, double G, double res,
                                double k_r_k_s, double k_t_k_s, double mu_s, double mu_r,
                                double mu_t);                                                 /* dataBase.h:111 */
DEMSPH_API int demsph_builder_set_linear(demsph_builder* b, int mi, int mj, double k_n, double k_s, double k_r,
                              double k_t, double d_n, double d_s, double d_r, double d_t, double mu_s,
                              double mu_r, double mu_t);                                      /* dataBase.h:130 */
DEMSPH_API int demsph_builder_set_bonded(demsph_builder* b, int mi, int mj, double E, double k_n_k_s, double gamma,
                              double sigma_s, double C, double mu);                           /* dataBase.h:152 */
DEMSPH_API int demsph_builder_add_fluid(demsph_builder* b, int n, const double* xyz, const double velocity[3],
                             double smoothing_length, double density, double sound_speed,
                             double kinematic_viscosity);                                     /* dataBase.cpp:3 */
DEMSPH_API int demsph_builder_add_dummy_wall(demsph_builder* b, int n, const double* xyz, double spacing); /* dataBase.cpp:19 */
DEMSPH_API int demsph_builder_add_solid(demsph_builder* b, int n, const double* xyz, const double velocity[3],
                             double radius, double density, int material);                    /* dataBase.cpp:33 */
DEMSPH_API int demsph_builder_add_infinite_wall(demsph_builder* b, const double point[3], const double normal[3],
                                     int material);                                           /* dataBase.cpp:55 */
DEMSPH_API int demsph_builder_add_cylinder_wall(demsph_builder* b, const double point[3], const double axis[3],
                                     const double angular_velocity[3], double radius, int material); /* dataBase.cpp:69 */
DEMSPH_API int demsph_builder_add_cluster(demsph_builder* b, int n, const double* xyz, const double* radius,
                               const double* density, const double velocity[3], int material); /* dataBase.cpp:84 */
DEMSPH_API int demsph_builder_add_clump(demsph_builder* b, int n, const double* xyz, const double* radius,
                             const double centroid[3], const double velocity[3],
                             const double angular_velocity[3], double mass, const double inertia6[6],
                             int material);                                                   /* dataBase.cpp:120 */
/* Points *out at the builder's arrays (valid until the builder changes or is freed). */
DEMSPH_API int demsph_builder_scene(const demsph_builder* b, demsph_scene* out);

/* ---- engine life cycle ---- */
/* DeviceData::copy of every part + dataBase::setSpatialGrids/buildDeviceData
   (core/dataBase.cpp:415-449).  opts may be NULL (defaults). */
DEMSPH_API int demsph_create(const demsph_scene* scene, const demsph_options* opts, demsph_engine** out);
/* DeviceData::release (core/deviceStructs.h:1033-1048). */
DEMSPH_API int demsph_destroy(demsph_engine* e);
/* Device part of solverBase::initialize (core/solverBase.cpp:29-31):
   neighborSearch(dev, 0, 1), addBondData (core/dataBase.cpp:270-346) and
   setSolidNormal (core/dataBase.cpp:348-413), all on the GPU. */
DEMSPH_API int demsph_initialize(demsph_engine* e);

/* ---- the five step functions (one call each per solverBase::update) ---- */
DEMSPH_API int demsph_neighbor_search(demsph_engine* e, int i_step, int gap);               /* neighborSearch.cu:314-382 */
DEMSPH_API int demsph_solid_integrate_before_contact(demsph_engine* e, double dt);          /* integrate.cu:964-980 */
DEMSPH_API int demsph_fluid_integrate(demsph_engine* e, double dt, int i_step, int gap);    /* integrate.cu:385-421 */
DEMSPH_API int demsph_solid_contact_after_fluid_integrate(demsph_engine* e, double dt);     /* integrate.cu:940-962 */
DEMSPH_API int demsph_solid_integrate_after_contact(demsph_engine* e, double dt);           /* integrate.cu:982-998 */
/* n_steps consecutive solverBase::update() bodies (core/solverBase.cpp:47-58)
   for i_step = first_step .. first_step+n_steps-1, without the driver hook;
   replayed as a CUDA graph when use_graph != 0. */
DEMSPH_API int demsph_update(demsph_engine* e, double dt, int first_step, int n_steps, int gap, int use_graph);
/* demsph_update for callers that exchange the state with the host every call
   (a coupled external solver): uploads the given host arrays (FP64, the
   layouts of demsph_upload_fluids / demsph_upload_solids; NULL = keep),
   advances the steps, downloads into the given host arrays (the layouts of
   demsph_download_fluids / demsph_download_solids; NULL = skip), and
   synchronises once at the end (and once after the upload when solid
   velocities are given in a scene with dummy particles: see
   demsph_upload_solids).  A list overflow is handled as in demsph_update
   (the transfer out follows the completed steps).  No counterpart in the
   reference. */
DEMSPH_API int demsph_update_io(demsph_engine* e, double dt, int first_step, int n_steps, int gap, int use_graph,
                                const double* fluid_pos_in, const double* fluid_vel_in, const double* fluid_drho_in,
                                const double* solid_pos_in, const double* solid_vel_in, const double* solid_angvel_in,
                                double* fluid_pos_out, double* fluid_vel_out, double* fluid_drho_out,
                                double* solid_pos_out, double* solid_vel_out, double* solid_angvel_out);
/* Chooses the threads per fluid particle of the fluid list and pair kernels
   (1, 2, 4 or 8) by timing the first continuity pass with each; call after
   demsph_initialize.  *lanes_out receives the choice (may be NULL).  No
   counterpart in the reference. */
DEMSPH_API int demsph_autotune(demsph_engine* e, int* lanes_out);
/* Launch shapes in use (no counterpart in the reference, whose kernels use fixed
   block sizes): threads per fluid particle, threads per clump, and contact rows
   per warp of the contact-force kernel; whether the fluid lists are kept as
   membership bits (DEMSPH_FLUID_TILES=1 at creation) and their words per
   fluid particle (both 0 with the list kernels). */
typedef struct demsph_launch_shapes {
    int fluid_lanes;
    int clump_lanes;
    int contact_force_rows;
    int fluid_bit_lists;
    int fluid_bit_words;
} demsph_launch_shapes;
DEMSPH_API int demsph_get_launch_shapes(const demsph_engine* e, demsph_launch_shapes* out);
/* Counters of the engine's update runs since creation (no counterpart in the
   reference): list growths after an overflow, steps resumed from their
   midpoint (their opening half step had run, in a pass that also closed the
   step before, when the neighbour search overflowed), and integration passes
   that closed one step and opened the next. */
typedef struct demsph_run_stats {
    long long list_growths;
    long long resumed_steps;
    long long fused_passes;
} demsph_run_stats;
DEMSPH_API int demsph_get_run_stats(const demsph_engine* e, demsph_run_stats* out);
/* The CUDA stream (cudaStream_t) the engine issues all its work on, for
   callers that time or order work around it. */
DEMSPH_API void* demsph_stream(demsph_engine* e);
/* Device memory the engine holds now (bytes), and an estimate, before
   creation, of what demsph_create will allocate for a scene (without later
   list growth or bonds).  No counterpart in the reference, whose memory is
   sized by dataBase on the host. */
DEMSPH_API long long demsph_device_bytes(const demsph_engine* e);
DEMSPH_API long long demsph_estimate_bytes(const demsph_scene* scene, const demsph_options* opts);
/* Kernels this engine has executed so far (graph replays counted by their
   kernels), as issued from the calling thread. */
DEMSPH_API long long demsph_kernel_launches(demsph_engine* e);
/* Per-stage timing with CUDA events on the engine's stream (enable != 0).
   While enabled, demsph_update runs uncaptured so every launch is timed. */
DEMSPH_API int demsph_set_profiling(demsph_engine* e, int enable);
/* Writes "name launches total_ms\n" lines for the stages timed since the last
   report into buf (NUL-terminated, truncated to cap) and resets the tally. */
DEMSPH_API int demsph_profile_report(demsph_engine* e, char* buf, int cap);
/* Waits for queued work; returns the first deferred error (e.g. capacity). */
DEMSPH_API int demsph_synchronize(demsph_engine* e);

/* ---- state transfer (fluid/solid/clump uploadState, core/deviceStructs.h) ---- */
DEMSPH_API int demsph_download_fluids(demsph_engine* e, double* position, double* velocity, double* acceleration,
                           double* drho);
DEMSPH_API int demsph_download_solids(demsph_engine* e, double* position, double* velocity, double* acceleration,
                           double* normal, double* torque, double* angular_velocity);
DEMSPH_API int demsph_download_clumps(demsph_engine* e, double* centroid, double* velocity, double* acceleration,
                           double* angular_velocity, double* torque, double* orientation);
/* Overwrite the dynamic state (inverse of the downloads); NULL skips a field.
   A dummy particle given a non-zero velocity is integrated from then on (and
   no longer once its velocity is zero again): the device compares the
   uploaded velocities with the dummy particles' current motion and the call
   waits for that one word before it returns. */
DEMSPH_API int demsph_upload_fluids(demsph_engine* e, const double* position, const double* velocity, const double* drho);
DEMSPH_API int demsph_upload_solids(demsph_engine* e, const double* position, const double* velocity,
                         const double* angular_velocity);

/* ---- run-time setters of class dataBase ---- */
DEMSPH_API int demsph_set_gravity(demsph_engine* e, const double g[3]);                              /* dataBase.h:105-109 */
DEMSPH_API int demsph_set_contact_models(demsph_engine* e, const demsph_scene* tables);              /* dataBase.h:111-167 */
DEMSPH_API int demsph_set_clump_velocity(demsph_engine* e, int clump, const double v[3]);            /* dataBase.h:169-182 */
DEMSPH_API int demsph_add_external_force(demsph_engine* e, int solid, const double force[3]);        /* dataBase.cpp:179-195 */
DEMSPH_API int demsph_add_global_damping(demsph_engine* e, int solid, double c_d);                   /* dataBase.cpp:197-224 */

/* ---- frame files of class solverBase (core/solverBase.cpp:69-333) ----
   <dir>/fluid_NNNN.vtu, solid_NNNN.vtu and fluid2Solid_NNNN.vtu with the
   reference's arrays, names and order, written as binary VTU (appended raw
   data, UInt64 headers) instead of ASCII.  A write packs the frame's FP32
   arrays on the engine's stream and returns; a background thread of the
   writer copies them into pinned memory and writes the files while the
   following steps run.  Each kind keeps two frames in flight: a write waits
   while the file of the same kind two frames back is not yet written.  The
   static arrays (smoothing length, radius, clusterID, clumpID) are taken from
   `scene` (the engine's scene) at open.  fluid2Solid forces are the per-pair
   coupling forces of the last step when the engine keeps them (options.debug
   bit 0), else zeros.  Close the writer before destroying its engine; after
   demsph_append a write returns DEMSPH_ERR_STATE (open a new writer).  Errors
   of the writer thread are returned by the next write, flush or close
   (DEMSPH_ERR_IO, message in demsph_last_error of the engine). */
typedef struct demsph_frame_writer demsph_frame_writer;
#define DEMSPH_FRAME_FLUID 1          /* outputFluidVTU       (core/solverBase.cpp:69-170) */
#define DEMSPH_FRAME_SOLID 2          /* outputSolidVTU       (core/solverBase.cpp:172-257) */
#define DEMSPH_FRAME_FLUID2SOLID 4    /* outputFluid2SolidVTU (core/solverBase.cpp:259-333) */
#define DEMSPH_FRAME_ALL 7
DEMSPH_API int demsph_frame_writer_open(demsph_engine* e, const demsph_scene* scene, const char* dir,
                                        demsph_frame_writer** out);
/* Enqueues the files of the kinds in `what` for frame number `frame` (the
   NNNN of the names), with TIME and STEP field data. */
DEMSPH_API int demsph_frame_writer_write(demsph_frame_writer* w, int what, int frame, int step, double time);
/* Waits until every enqueued file is written. */
DEMSPH_API int demsph_frame_writer_flush(demsph_frame_writer* w);
/* Flushes, stops the thread and frees the writer (also after an error). */
DEMSPH_API int demsph_frame_writer_close(demsph_frame_writer* w);

/* ---- particles added while the simulation runs ----
   dataBase::addFluid / addSolid / addCluster / addDummyParticleWall after the
   start (dataBase::addFluidData / addSolidData with iStep > 0,
   core/dataBase.cpp:226-268; addCluster's search and bonds, :83-113 and
   :307-343).  `current` is the scene as it stands - its parameters, its
   contact tables and its clump and wall data (the dynamic state is taken from
   the engine); `additions` holds the new fluids and solids (no walls and no
   clumps: DEMSPH_ERR_ARGUMENT, as the reference refuses walls after the
   start).  They follow the old particles in index order.  As in the
   reference: the spatial grid is recomputed, the contact springs carry over,
   wall springs start from zero, new solids have zero normals, and a new
   cluster is bonded above the last bonded solid.  Unlike the reference: the
   lists are searched at once (the reference searches at the next step, or at
   once for a cluster), and new fluids take their Shepard reference sums at
   the append (the reference leaves them zero and divides by them at its next
   re-initialisation).  The handle stays valid; the engine behind it is new
   (graphs are captured again). */
DEMSPH_API int demsph_append(demsph_engine* e, const demsph_scene* current, const demsph_scene* additions);

/* ---- artefacts in the reference's index space and order (for parity) ---- */
DEMSPH_API int demsph_get_counts(demsph_engine* e, demsph_counts* out);
/* objectHash after buildHashSpans (core/neighborSearch.cu:71-113): per particle
   the cell key (hash.value, sorted) and the sorted particle index (hash.index),
   and cellStart/cellEnd per cell (-1 = empty).  which: 0 fluid, 1 solid. */
DEMSPH_API int demsph_export_cell_hash(demsph_engine* e, int which, int* hash_value, int* hash_index, int* cell_start,
                            int* cell_end);
/* fluid2Fluid half list (core/neighborSearch.cu:115-220): prefix = inclusive
   prefix sum per fluid particle; pairs in the reference's order. */
DEMSPH_API int demsph_export_fluid_pairs(demsph_engine* e, int* prefix, int* pointed, int* pointing, long long capacity);
/* fluid2Solid list and the per-pair coupling force (core/integrate.cu:282-330). */
DEMSPH_API int demsph_export_fluid_solid_pairs(demsph_engine* e, int* prefix, int* pointed, int* pointing, double* force,
                                    long long capacity);
/* solid2Solid half list with forces, torques and springs
   (core/neighborSearch.cu:222-312, core/integrate.cu:423-512). */
DEMSPH_API int demsph_export_solid_pairs(demsph_engine* e, int* prefix, int* pointed, int* pointing, double* force,
                              double* torque, double* sliding, double* rolling, double* torsion,
                              long long capacity);
/* interactionBonded (core/deviceStructs.h:714-789). */
DEMSPH_API int demsph_export_bonds(demsph_engine* e, int* pointed, int* pointing, int* is_bonded, double* normal_force,
                        double* torsion_torque, double* shear_force, double* bending_torque,
                        double* contact_normal, double* contact_point, long long capacity);
/* Conservation audit, summed in FP64 on the GPU: mass, linear momentum,
   translational kinetic energy, rotational kinetic energy of spheres (clumps
   as rigid bodies, translation only), potential energy -m g.x (x from the
   domain origin) and the sum of fluid densities.  Fluids, solids with mass
   and clumps; dummy and fixed particles carry none.  No counterpart in the
   reference. */
typedef struct demsph_audit_values {
    double mass;
    double momentum[3];
    double kinetic_energy;
    double rotational_energy;
    double potential_energy;
    double fluid_density_sum;
} demsph_audit_values;
DEMSPH_API int demsph_audit(demsph_engine* e, demsph_audit_values* out);

/* Shepard reference sums sumW0 (core/integrate.cu:44-47). */
DEMSPH_API int demsph_export_fluid_sumw0(demsph_engine* e, double* sumw0);

/* ---- many scenes in one graph launch ----
   No counterpart in the reference (one scene per process).  One call advances
   engines[0..count) by n_steps[k] steps from first_step[k] each (time step
   dt[k], fluid gap gap[k]), all in one CUDA graph launch: each engine's round
   of steps is a child graph, captured once per (phase in the fluid and
   Shepard schedule, length, contact-list parity, dt, gap), the children run as
   independent branches, and the executable graph is reused while every
   member's round repeats (rounds of even length that are multiples of
   5 gap steps repeat).  Every scene's state afterwards is bit for bit its state
   after demsph_update over the same steps.  Step 1 and profiled runs go
   through demsph_update first; a member whose lists overflowed grows them and
   finishes its steps alone before the call returns.  status_out[k] receives
   each engine's status (its message in demsph_last_error); the return value
   is DEMSPH_OK unless the launch itself failed.  All engines on the batch's
   device; none may be used by another thread during the call. */
typedef struct demsph_batch demsph_batch;
typedef struct demsph_batch_info {
    long long launches;      /* graph launches so far */
    long long graph_builds;  /* executable graphs instantiated (member rounds changed) */
    long long members;       /* engines in the last built graph */
    long long nodes;         /* nodes in it */
    double capture_s;        /* host time spent capturing members' rounds */
    double instantiate_s;    /* host time spent building and instantiating the batch graphs */
    double launch_s;         /* host time from each launch to its completion */
} demsph_batch_info;
DEMSPH_API int demsph_batch_create(int device, demsph_batch** out);
DEMSPH_API int demsph_batch_destroy(demsph_batch* b);
DEMSPH_API int demsph_batch_update(demsph_batch* b, demsph_engine* const* engines, int count, const int* first_step,
                                   const int* n_steps, const double* dt, const int* gap, int* status_out);
DEMSPH_API int demsph_batch_get_info(const demsph_batch* b, demsph_batch_info* out);
DEMSPH_API const char* demsph_batch_last_error(const demsph_batch* b);

/* ---- scene server: many scenes on one GPU ----
   No counterpart in the reference (one scene per process).  Scenes are
   submitted with a step count, admitted first come, first served while their
   estimated device memory fits the budget, and advanced together - each on
   its own engine and CUDA stream, in chunks of steps replayed from CUDA graphs, by a
   pool of worker threads - so that scenes arriving while others run join as
   memory frees up.  Results stay on the host until released. */
typedef struct demsph_server demsph_server;
typedef struct demsph_server_config {
    int device;                  /* CUDA device ordinal */
    int workers;                 /* host threads advancing scenes; 0 = 8 */
    int chunk_steps;             /* steps per turn of a scene; 0 = 100 */
    long long hbm_budget_bytes;  /* device memory the admitted scenes may hold; 0 = 150 GiB */
    int autotune;                /* != 0: the first scene of each size class (fluid count within a
                                    factor of 2) runs demsph_autotune, later ones reuse its choice */
    int graphs;                  /* CUDA graphs for a turn: 0 = only when the scene is the only
                                    active one (default), 1 = always, -1 = never.  Capturing and
                                    instantiating graphs while other scenes' kernels run was measured
                                    hundreds of times slower than on an idle GPU, so scenes in a mix
                                    launch their kernels directly (the same results, bit for bit) */
    int batch;                   /* != 0: one host thread advances all active scenes together, each
                                    round one demsph_batch_update launch (rounds of about
                                    batch_round_steps steps, whole Shepard periods); workers then
                                    only create engines and download results */
    int batch_round_steps;       /* 0 = 20 */
} demsph_server_config;
typedef struct demsph_server_summary {
    long long submitted, admitted, completed, failed, pending;
    long long steps;             /* scene steps run */
    long long particle_updates;  /* fluid particles per fluid step + solids with mass per step */
    long long chunks;            /* turns taken (latency samples) */
    long long bytes_in_use, peak_bytes;  /* reserved against the budget */
    double busy_s;               /* first admission to the last completion (or now) */
    double updates_per_s;        /* particle_updates / busy_s */
    double p50_step_ms, p99_step_ms;     /* wall time per scene step, queueing for the GPU included */
    double create_s, step_s, download_s; /* worker time summed over workers: engine creation and
                                            initialisation, stepping, downloading results */
    long long batch_rounds, batch_graph_builds;    /* batch mode: launches, graphs instantiated */
    double batch_capture_s, batch_instantiate_s, batch_launch_s;  /* batch mode: time in each */
} demsph_server_summary;
typedef struct demsph_request_info {
    int state;                   /* 0 pending, 1 running, 2 done, 3 failed */
    int steps_done;
    long long reserved_bytes;
    double queued_s, run_s;
} demsph_request_info;
DEMSPH_API int demsph_server_create(const demsph_server_config* cfg, demsph_server** out);
DEMSPH_API int demsph_server_destroy(demsph_server* s);
/* Copies the scene; steps 1..n_steps of solverBase::update follow
   (scene->time_step, scene->fluid_integrate_gap).  DEMSPH_ERR_CAPACITY: the
   scene alone exceeds the budget. */
DEMSPH_API int demsph_server_submit(demsph_server* s, const demsph_scene* scene, const demsph_options* opts,
                                    int n_steps, long long* request_id);
/* Waits until the request (or, for id -1, every request) has finished;
   timeout_s < 0 waits without limit.  Returns the request's status. */
DEMSPH_API int demsph_server_wait(demsph_server* s, long long request_id, double timeout_s);
/* Final state of a finished request (original order, FP64, 3 per particle;
   dRho 1 per particle); NULL skips an array. */
DEMSPH_API int demsph_server_fetch(demsph_server* s, long long request_id, double* fluid_position,
                                   double* fluid_velocity, double* fluid_drho, double* solid_position,
                                   double* solid_velocity, double* solid_angular_velocity);
DEMSPH_API int demsph_server_release(demsph_server* s, long long request_id);
DEMSPH_API int demsph_server_request_info(demsph_server* s, long long request_id, demsph_request_info* info);
DEMSPH_API int demsph_server_stats(demsph_server* s, demsph_server_summary* stats);

/* ---- cell sort without allocation ----
   No counterpart in the reference.  Sorts n particle cell keys (device
   array, each in [0, num_cells)) by (key, original index): sorted_index[n]
   receives the original indices in that order, cell_start / cell_end
   [num_cells] the first and one-past-last position of each cell in it (-1
   for an empty cell); all three are device arrays.  For callers that cannot
   allocate device memory when they call it (their own allocator already
   holds the GPU's memory, or they must avoid cudaMalloc's synchronisation):
   the scratch is one fixed array of device memory in this library, about
   8 MB, that every GPU loading the library keeps until exit.  Limits: n and
   num_cells at most 524288 each; larger sizes return DEMSPH_ERR_ARGUMENT, as
   do keys outside [0, num_cells) (those elements are left out).  Ordering a
   cell costs each of its elements one pass over the cell: meant for particle
   cell keys, tens per cell.  The first call on each device (and CUDA
   context) looks up the array's address there; make that first call before
   any stream capture.  All calls share the array: calls that overlap on the
   GPU (other streams, other threads) race and must be serialised by the
   caller.  The call reads a flag back to the host and waits for its stream.
   stream is a cudaStream_t (NULL = the default stream). */
DEMSPH_API int demsph_cell_sort_noalloc(const int* keys, int n, int num_cells, int* sorted_index, int* cell_start,
                                        int* cell_end, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* DEMSPH_GB300_H */
