/*
 * spacecharge_gb300.h — C ABI of the GB300 space-charge kick library
 * (libspacecharge_gb300.so).
 *
 * The library replaces the hot path of SpaceCharge.jl v1.2.0:
 *   Mesh3D (src/mesh.jl:95-238) -> deposit! (src/deposition.jl:218)
 *   -> solve! (src/solvers/free_space.jl:14) -> interpolate_field
 *   (src/interpolation.jl:100).
 * A Julia host binds these functions with `ccall`; the Python host in
 * spacecharge.jl_gb300/python binds them with ctypes.
 *
 * Conventions
 *  - Every function returns an int status (SC_OK = 0).  On failure
 *    sc_last_error() returns a message for the calling thread.  Argument
 *    errors that the reference raises with `error("...")` return
 *    SC_ERR_INVALID with the reference's message text.
 *  - Particle arrays and field outputs are DEVICE pointers (CuArray /
 *    torch CUDA storage) of `dtype` (SC_F32 or SC_F64); outputs have the
 *    particle dtype, as `similar(particles_x)` does (interpolation.jl:110).
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Work is
 *    enqueued asynchronously; nothing synchronises unless stated.
 *  - Arrays are column-major as in Julia: rho is (nx,ny,nz) with x fastest.
 *    efield is (nx,ny,nz,3) component-planar for SC_PREC_PLAIN64 meshes and
 *    packed (4,nx,ny,nz) = (Ex,Ey,Ez,0) per node for the hand-written
 *    pipelines (sc_mesh_info.efield_layout says which).
 *  - Threads: different meshes (and batches) may be used from different
 *    host threads at once; one mesh is used by one thread at a time, as a
 *    Julia Mesh3D is (its fields and workspace are mutated in place).
 */
#ifndef SPACECHARGE_GB300_H
#define SPACECHARGE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SC_OK               0
#define SC_ERR_INVALID      1  /* bad argument (the reference's ErrorException) */
#define SC_ERR_CUDA         2  /* CUDA runtime / cuFFT failure */
#define SC_ERR_OOM          3  /* device allocation failed */
#define SC_ERR_OUT_OF_RANGE 4  /* particles outside the mesh were skipped */
#define SC_ERR_TIMEOUT      5  /* a bounded device-side wait gave up */
#define SC_ERR_UNSUPPORTED  6  /* size or option the library does not handle */

/* particle / output element types */
#define SC_F32 0
#define SC_F64 1

/* mesh precision (the Julia wrapper maps T=Float64 -> SC_PREC_FP64,
 * T=Float32 -> SC_PREC_MIXED) */
#define SC_PREC_PLAIN64 0 /* the reference algorithm, FP64, cuFFT Z2Z, 7 FFTs */
#define SC_PREC_FP64    1 /* hand-written pruned pipeline in FP64 */
#define SC_PREC_MIXED   2 /* hand-written pipeline: FP32 deposit/FFT/gather,
                             FP64 IGF differences, origin offsets, charge sum */

/* deposit modes */
#define SC_DEPOSIT_ATOMIC        0 /* one thread per particle, 8 atomics */
#define SC_DEPOSIT_SORTED        1 /* bin by cell, warp-segmented sums, few atomics */
#define SC_DEPOSIT_DETERMINISTIC 2 /* sorted, fixed-point sums: bitwise reproducible */
#define SC_DEPOSIT_TILED         3 /* sorted by 8x8x8-cell tile, shared-memory accumulation */
#define SC_DEPOSIT_VECTOR        4 /* mixed meshes: two 16-byte vector atomics per particle
                                      into per-cell corners, then a node sum; on FP64
                                      meshes the same as SC_DEPOSIT_ATOMIC */

/* pipeline stages timed by sc_mesh_stage_times */
#define SC_STAGE_DEPOSIT   0 /* clear + deposit kernels */
#define SC_STAGE_GREEN     1 /* Green-function build (IGF + its transform) */
#define SC_STAGE_FWD_X     2 /* hand-written: real rows -> half spectra */
#define SC_STAGE_FWD_Y     3 /* hand-written: y transform */
#define SC_STAGE_ZPASS     4 /* hand-written: z transform x Green x inverse z */
#define SC_STAGE_INV_Y     5 /* hand-written: inverse y */
#define SC_STAGE_INV_X     6 /* hand-written: inverse x -> packed efield */
#define SC_STAGE_GATHER    7 /* interpolation */
#define SC_STAGE_PLAIN_FFT 8 /* plain path: pad, cuFFT Z2Z, product, extract */
#define SC_NUM_STAGES      9

/* efield layouts */
#define SC_LAYOUT_PLANAR 0
#define SC_LAYOUT_PACKED 1

typedef struct sc_mesh sc_mesh;

typedef struct sc_mesh_info {
    int32_t grid_size[3];
    int32_t precision;
    double  min_bounds[3];
    double  max_bounds[3];
    double  delta[3];
    double  gamma;
    double  total_charge;
    int32_t efield_layout;  /* SC_LAYOUT_* */
    int32_t elem_bytes;     /* sizeof element of rho / efield */
    int32_t fft_shape[3];   /* transform length per axis */
    int32_t device;
} sc_mesh_info;

/* Library version (major*10000 + minor*100 + patch). */
int sc_version(void);

/* Message of the last failing call on this thread ("" if none). */
const char* sc_last_error(void);

/* Manual-bounds constructor: Mesh3D(grid_size, min_bounds, max_bounds;
 * T, gamma, total_charge), src/mesh.jl:196-238.  Validates grid >= 2 and
 * max > min (mesh.jl:206-211); delta = (max-min)/(n-1) (mesh.jl:220).
 * Allocates rho and efield (zeroed) on the current CUDA device. */
int sc_mesh_create(const int32_t grid_size[3], const double min_bounds[3],
                   const double max_bounds[3], double gamma, double total_charge,
                   int precision, sc_mesh** out);

/* The bounds arithmetic of the particle-bounds constructor, src/mesh.jl:
 * 106-150: validation, extrema (one device reduction + a 48-byte copy to
 * the host, which synchronises `stream`), 1e-6*delta padding, delta
 * recomputation and the delta == 0 -> 1e-6 patch, all in FP64. */
int sc_auto_bounds(const int32_t grid_size[3], const void* x, const void* y,
                   const void* z, int64_t n, int dtype, double min_bounds[3],
                   double max_bounds[3], double delta[3], void* stream);

/* The same bounds from extrema the caller already has (for instance reduced
 * over the ranks that each hold part of a bunch): the padding and delta
 * arithmetic of mesh.jl:125-150 on mins[3], maxs[3].  Host only. */
int sc_bounds_from_extrema(const int32_t grid_size[3], const double mins[3], const double maxs[3],
                           double min_bounds[3], double max_bounds[3], double delta[3]);

/* Particle-bounds constructor: Mesh3D(grid_size, px, py, pz; T, gamma,
 * total_charge), src/mesh.jl:95-174.  Synchronises `stream`. */
int sc_mesh_create_from_particles(const int32_t grid_size[3], const void* x,
                                  const void* y, const void* z, int64_t n, int dtype,
                                  double gamma, double total_charge, int precision,
                                  void* stream, sc_mesh** out);

/* Frees the mesh, its fields and its workspace. */
int sc_mesh_destroy(sc_mesh* mesh);

/* New bounds for an existing mesh, keeping its grid, fields and workspaces
 * (no counterpart in the reference, whose Mesh3D geometry is set once; a
 * tracking code there builds a new mesh per step).  The validation and delta
 * of the manual constructor (src/mesh.jl:206-220).  Cached Green spectra and
 * captured kick graphs follow the new geometry on the next call. */
int sc_mesh_set_bounds(sc_mesh* mesh, const double min_bounds[3], const double max_bounds[3]);

/* The same with the particle constructor's bounds for x, y, z (sc_auto_bounds,
 * src/mesh.jl:95-174).  Synchronises `stream`. */
int sc_mesh_refit(sc_mesh* mesh, const void* x, const void* y, const void* z, int64_t n, int dtype,
                  void* stream);

/* Mesh properties (the fields of Mesh3D, src/mesh.jl:19-34). */
int sc_mesh_get_info(const sc_mesh* mesh, sc_mesh_info* info);

/* Device pointers to mesh.rho and mesh.efield (owned by the mesh). */
int sc_mesh_rho(sc_mesh* mesh, void** dptr);
int sc_mesh_efield(sc_mesh* mesh, void** dptr);

/* Enable (1, default) or disable (0) reuse of the Green-function spectrum
 * between solves while delta, gamma and the cathode offset are unchanged.
 * The reference rebuilds it on every solve! (free_space.jl:77-96). */
int sc_mesh_set_green_cache(sc_mesh* mesh, int enabled);

/* Arithmetic of an SC_PREC_FP64 mesh's kick (no counterpart in the
 * reference).  SC_FP64_ARITH_FP64 (default): FP64 throughout.
 * SC_FP64_ARITH_DF32: the atomic deposit's weights, the x and y transform
 * passes, the z pass (forward z transform, Green products, three inverse z
 * transforms; free space), the trilinear interpolation and the free-space
 * Green function's transform carry each value as the unevaluated sum of two
 * FP32 numbers (48-bit significands, FP32's exponent range, magnitudes from
 * 2^-103 to 2^128), with FP64 inputs and outputs; fields move by about
 * 1e-14 of their maximum.  The GB300 runs FP64 at 1/64 of its FP32 rate, so
 * this takes those passes off the FP64 units.  The Green function's corner
 * antiderivative stays FP64; meshes with a transform above 256 points keep
 * FP64 transforms, and the field's z pass with the cathode image stays FP64.
 * sc_solve_potential follows the mode too (its forward, z and inverse
 * passes, and its Green transform; the antiderivative stays FP64).  Other
 * precisions: SC_ERR_INVALID. */
#define SC_FP64_ARITH_FP64 0
#define SC_FP64_ARITH_DF32 1
int sc_mesh_set_fp64_arithmetic(sc_mesh* mesh, int mode);

/* FFT kernels of the hand-written pipelines (process-wide).  SC_FFT_AUTO
 * (default): register-resident two-step transforms for FP32 lengths up to
 * 256 (and for the double-FP32 z pass, sc_mesh_set_fp64_arithmetic),
 * shared-memory Stockham transforms otherwise; SC_FFT_STOCKHAM: the Stockham
 * transforms everywhere.  Both give the same result to rounding. */
#define SC_FFT_AUTO     0
#define SC_FFT_STOCKHAM 1
int sc_set_fft_engine(int engine);

/* Test hook for the error paths (no counterpart in the reference): after
 * `after` more successful device allocations, every allocation the library
 * makes fails with SC_ERR_OOM, without calling the runtime, until a negative
 * `after` switches the injection off.  Process-wide.  A call that fails this
 * way leaves its mesh usable: the next call with allocations allowed
 * retries them. */
int sc_test_fail_allocations(int64_t after);

/* clear_mesh!(mesh), src/deposition.jl:10-12. */
int sc_clear_mesh(sc_mesh* mesh, void* stream);

/* deposit!(mesh, px, py, pz, pq; clear), src/deposition.jl:218-247.
 * Cell indices are floor((x - min)/delta) in FP64 exactly as the
 * reference computes them (deposition.jl:39-46).  Particles whose cell is
 * outside the mesh are skipped and counted (the reference has no check,
 * deposition.jl:64); read the count with sc_mesh_out_of_range. */
int sc_deposit(sc_mesh* mesh, const void* x, const void* y, const void* z,
               const void* q, int64_t n, int dtype, int clear, int mode, void* stream);

/* Deposit mode sc_kick uses for this mesh (default SC_DEPOSIT_VECTOR for
 * SC_PREC_MIXED, SC_DEPOSIT_ATOMIC otherwise).  With SC_DEPOSIT_TILED the
 * kick also gathers through the same tiles.  SC_PREC_PLAIN64 meshes always
 * kick with the atomic deposit. */
int sc_mesh_set_kick_mode(sc_mesh* mesh, int mode);

/* sc_kick with the particles and outputs in HOST memory (no counterpart in
 * the reference, whose arrays are CuArrays).  The library copies the
 * particles to its own device buffers in chunks on a copy stream,
 * depositing each chunk as it arrives, and copies each chunk's field back
 * while the next is gathered.  Page-locked host buffers give the overlap;
 * pageable ones work but copy synchronously.  The outputs are valid once
 * `stream` has reached this call's end.  The sorted, deterministic and tiled
 * kick modes copy everything first. */
int sc_kick_host(sc_mesh* mesh, const void* x, const void* y, const void* z, const void* q, int64_t n, int dtype,
                 int at_cathode, void* ex, void* ey, void* ez, void* stream);

/* Graph replay of sc_kick (default on; no counterpart in the reference).  A
 * call with the same particle and output pointers, count, dtype and cathode
 * flag as the previous one, on an unchanged mesh, replays a CUDA graph of the
 * kick (one launch on the caller's stream).  The first call with new
 * arguments runs the kick eagerly and then captures it.  Kicks with stage
 * profiling on, on SC_PREC_PLAIN64 meshes, or issued into a stream that is
 * being captured run eagerly. */
int sc_mesh_set_kick_graph(sc_mesh* mesh, int enabled);

/* solve!(mesh; at_cathode), src/solvers/free_space.jl:14-101. */
int sc_solve(sc_mesh* mesh, int at_cathode, void* stream);

/* interpolate_field(mesh, px, py, pz) -> (Ex, Ey, Ez),
 * src/interpolation.jl:100-128, into caller-owned device outputs. */
int sc_interpolate_field(sc_mesh* mesh, const void* x, const void* y, const void* z,
                         int64_t n, int dtype, void* ex, void* ey, void* ez,
                         void* stream);

/* deposit! + solve! + interpolate_field in one call: the unit timed by
 * benchmark/full_pipeline_benchmark.jl:43-48. */
int sc_kick(sc_mesh* mesh, const void* x, const void* y, const void* z, const void* q,
            int64_t n, int dtype, int at_cathode, void* ex, void* ey, void* ez,
            void* stream);

/* The binning step of deposit!/interpolate_field on its own: for each
 * particle, the 0-based lower-corner node (ix, iy, iz) = floor((x-min)/delta)
 * (deposition.jl:39-46) into idx[3*p .. 3*p+2], or -1s when outside the
 * mesh, and the in-cell fractions (deposition.jl:49-51) into frac[3*p ..]
 * as FP64.  Uses the same device arithmetic as the mesh's deposit kernel. */
int sc_cell_index(sc_mesh* mesh, const void* x, const void* y, const void* z, int64_t n, int dtype,
                  int32_t* idx, double* frac, void* stream);

/* Stage timing: while enabled, every stage of deposit/solve/interpolate is
 * bracketed by CUDA events recorded on the caller's stream.
 * sc_mesh_stage_times synchronises `stream`, writes the milliseconds and the
 * number of timed executions per stage accumulated since the previous query
 * (arrays of SC_NUM_STAGES), and resets them. */
int sc_mesh_set_profiling(sc_mesh* mesh, int enabled);
int sc_mesh_stage_times(sc_mesh* mesh, double* ms, int64_t* calls, void* stream);

/* Number of kernels this mesh has launched since it was created (cuFFT's
 * internal kernels count as one per transform). */
int sc_mesh_launch_count(const sc_mesh* mesh, int64_t* count);

/* Hand-written adjoint of sc_kick (the pullback of the ChainRulesCore.rrule
 * of `kick` in the Julia host; the reference itself is not differentiable:
 * src/mesh.jl:100 restricts T to AbstractFloat).  Recomputes the forward
 * deposit and solve for these particles (mesh.rho / mesh.efield are left as
 * after sc_kick, except efield's unused fourth lane), then returns
 * d(loss)/d(x, y, z, q) into dx, dy, dz, dq (particle dtype) given
 *   gex, gey, gez : d(loss)/d(Ex, Ey, Ez) at the particles (NULL = zero),
 *   ggrid         : d(loss)/d(mesh.efield) in the mesh's packed layout
 *                   (4, nx, ny, nz) of its element type, or NULL.
 * The mesh geometry is held fixed; gradients are those of the piecewise
 * smooth map inside each particle's cell.  Needs an SC_PREC_FP64 or
 * SC_PREC_MIXED mesh (SC_ERR_UNSUPPORTED otherwise). */
int sc_kick_adjoint(sc_mesh* mesh, const void* x, const void* y, const void* z, const void* q, int64_t n,
                    int dtype, int at_cathode, const void* gex, const void* gey, const void* gez,
                    const void* ggrid, void* dx, void* dy, void* dz, void* dq, void* stream);

/* Allocation-free free-space solve.  This entry point has no counterpart in
 * the reference.  It is for callers that cannot let a library call
 * cudaMalloc: a host code that owns all device memory through its own pool,
 * or a loop that forbids device allocation once it is running.  It computes
 * the same field as sc_solve(at_cathode = 0) on an SC_PREC_MIXED mesh of
 * this grid, delta and gamma (Green function rebuilt on every call), from
 * the caller's rho (FP32, nx*ny*nz, x fastest) into the caller's efield
 * (FP32, packed (4, nx, ny, nz) = (Ex, Ey, Ez, 0) per node).  It calls no
 * cudaMalloc, cudaFree or allocating library routine: its workspace is one
 * file-scope device array of about 8.6 MB.  The array is committed on a
 * device when the library's kernels are loaded there (under CUDA's lazy
 * module loading, the default, at the library's first call on that device)
 * and is held until that device's context is destroyed.
 *  - Grids are limited to 32 nodes per axis; larger ones return
 *    SC_ERR_UNSUPPORTED with a message naming the limit.
 *  - The first call on a device uploads an 8 KB twiddle table into the
 *    array (a synchronous copy); make that first call before any stream
 *    capture.  Every call looks up the array's device address; after a
 *    device reset the array has a new one and the next call uploads the
 *    table again.
 *  - All calls on a device share the array and it keeps the last call's
 *    contents; calls that overlap on the GPU (other streams, other host
 *    threads) race and must be serialised by the caller. */
int sc_solve_noalloc(const int32_t grid_size[3], const double delta[3], double gamma, const float* rho,
                     float* efield, void* stream);

/* ---- many bunches: one call for their kicks, replayed as a CUDA graph ----
 * No counterpart in the reference (a tracking code calls its kick once per
 * bunch: benchmark/full_pipeline_benchmark.jl:64-71 times one at a time).
 * A batch references caller-owned meshes (SC_PREC_FP64 or MIXED, all on
 * the current device; each with its own grid, bounds and gamma).
 *  - Staged engine (default).  Bunches on SC_PREC_MIXED meshes with
 *    transforms of at most 256 points, Lx = Ly, and deposit mode
 *    SC_DEPOSIT_VECTOR or SC_DEPOSIT_ATOMIC are kicked stage by stage in
 *    groups (sc_batch_set_group_bytes): per group, on one internal stream
 *    (the first for every group when the call builds no Green spectrum;
 *    group g on stream g % nstreams when it does), one launch clears its
 *    bunches' charge buffers, one deposits them, one
 *    sums the corner slots, one or two run the forward x+y transforms
 *    (sc_batch_set_fused_forward), one the z pass with the Green multiply,
 *    one the inverse y+x pass and one the gather.  A vector-mode bunch with
 *    fewer particles than a quarter of its nodes deposits with scalar
 *    atomics instead.
 *  - The other bunches run their whole kick on internal stream
 *    i % nstreams, beside the groups.
 *  - The first call with a given set of pointers, counts, dtype and
 *    at_cathode plans the groups (synchronising `stream` once, allocating
 *    workspaces, building Green spectra, uploading the per-bunch tables),
 *    runs eagerly, and captures the same work into a CUDA graph; later
 *    calls with identical arguments replay the graph in one launch.  A
 *    planning call must not be issued while `stream` is being captured.
 *  - Meshes must not be destroyed while their batch exists. */
typedef struct sc_batch sc_batch;
int sc_batch_create(sc_mesh* const* meshes, int nbunch, int nstreams, sc_batch** out);
int sc_batch_kick(sc_batch* batch, const void* const* x, const void* const* y, const void* const* z,
                  const void* const* q, const int64_t* n, int dtype, int at_cathode, void* const* ex,
                  void* const* ey, void* const* ez, void* stream);
int sc_batch_set_graph(sc_batch* batch, int enabled); /* default 1 */
/* 0: every bunch on the per-bunch stream path (the staged engine off);
 * default 1. */
int sc_batch_set_staged(sc_batch* batch, int enabled);
/* Staged bunches are kicked in groups: consecutive bunches of one grid
 * class whose fields, charge buffers and transform intermediates together
 * take at most `bytes` (0: every bunch on its own, INT64_MAX: one group per
 * class).  Group g is one chain of stage launches on internal stream
 * g % nstreams, so a small budget keeps a group's data in L2 between its
 * stages and a large one saves launches.  The next kick plans anew. */
int sc_batch_set_group_bytes(sc_batch* batch, int64_t bytes);
/* 1: the staged forward x and y transforms as one fused pass per z plane;
 * 0: as an x pass and a y pass. */
int sc_batch_set_fused_forward(sc_batch* batch, int enabled);
/* Times graph replays of these kick arguments for group budgets of 0,
 * 48 MB, 128 MB, 512 MB and unbounded, each with the fused and the two-pass
 * forward transform, keeps the fastest for this batch and returns it in
 * *group_bytes and *fused_forward (either may be NULL).  Synchronising; the
 * arguments are sc_batch_kick's and are kicked 50 times. */
int sc_batch_autotune(sc_batch* batch, const void* const* x, const void* const* y, const void* const* z,
                      const void* const* q, const int64_t* n, int dtype, int at_cathode, void* const* ex,
                      void* const* ey, void* const* ez, void* stream, int64_t* group_bytes,
                      int* fused_forward);
/* Bunches the current plan kicks stage by stage, and the kernel launches
 * of those stages per kick (0 before the first kick). */
int sc_batch_staged_count(const sc_batch* batch, int* staged, int64_t* launches);
int sc_batch_graph_nodes(const sc_batch* batch, int64_t* count);
int sc_batch_destroy(sc_batch* batch);

/* FFT autotuner (no counterpart in the reference): times this mesh's solve
 * with each candidate kernel configuration -- the register two-step
 * transforms, and the Stockham transforms with 4, 8, 16 or 32 columns per
 * CTA -- and keeps the fastest for this mesh and for every later mesh with
 * the same transform shape and precision on this device.  When the
 * environment variable SC_AUTOTUNE_FILE names a file, choices are appended
 * to it and read back by later processes.  Synchronises `stream`; the
 * chosen configuration is written to *choice (0 = two-step, 2..5 = Stockham
 * with 2^choice columns) when choice is not NULL. */
int sc_autotune(sc_mesh* mesh, void* stream, int* choice);

/* Number of particles skipped as out of range since the last call
 * (deposit and interpolate); resets the counter.  Synchronises `stream`. */
int sc_mesh_out_of_range(sc_mesh* mesh, int64_t* count, void* stream);

/* ---- beside the kick (no counterpart in the reference) ---------------- */

/* Magnetic field of the bunch at the particles from its electric field
 * there, for a bunch moving along +z at the mesh's gamma:
 * B = (beta / c) z x E, i.e. Bx = -beta Ey / c, By = beta Ex / c, Bz = 0,
 * beta = sqrt(1 - 1/gamma^2).  Device arrays of the particle type. */
int sc_magnetic_field(const sc_mesh* mesh, const void* ex, const void* ey, int64_t n, int dtype, void* bx,
                      void* by, void* stream);

/* Array-of-structs particle records -> the SoA arrays the kick takes.
 * Record i starts at element i*stride; x, y, z, q sit at offs[0..3]. */
int sc_aos_to_soa(const void* aos, int64_t n, int stride, const int32_t offs[4], int dtype, void* x, void* y,
                  void* z, void* q, void* stream);

/* The kick's field components back into the records, at offs[0..2]. */
int sc_soa_to_aos(const void* ex, const void* ey, const void* ez, int64_t n, int dtype, int stride,
                  const int32_t offs[3], void* aos, void* stream);

/* FP32 positions relative to an FP64 reference point (e.g. the bunch
 * centroid) -> FP64 absolute positions x = ref + r (one rounding). */
int sc_relative_to_absolute(const float* rx, const float* ry, const float* rz, int64_t n, const double ref[3],
                            double* x, double* y, double* z, void* stream);

/* `steps` tracking steps of the bunch in its own field (the kick's caller
 * in a tracking code; no counterpart in the reference).  Each step: when
 * `refit`, new mesh bounds from the particles (the particle constructor's
 * arithmetic, mesh.jl:95-174; this synchronises), the kick, B = (beta/c)
 * z x E, and one relativistic Boris step of the dimensionless momenta
 * u = gamma*beta and the positions over `dt` seconds for a species of
 * charge/mass `qm` [C/kg].  x, y, z, ux, uy, uz are updated in place on the
 * device; q is the macro-particle charge [C].  Without `refit` the mesh keeps
 * its bounds and the kick replays its graph from the second step on. */
int sc_track(sc_mesh* mesh, void* x, void* y, void* z, void* ux, void* uy, void* uz, const void* q, int64_t n,
             int dtype, double dt, double qm, int steps, int refit, int at_cathode, void* stream);

/* Scalar potential on the mesh nodes from the deposited charge (the step
 * beside the field solve; the reference defines the potential
 * antiderivative, potential_green_function in green_functions.jl:13-22, but
 * never calls it).  The field solve's schedule (free_space.jl:14-101) with
 * that antiderivative and the transverse factor gamma/(dx dy dz): the
 * lab-frame potential gamma*phi' of the bunch's rest-frame potential.
 * `phi` is a device array of nx*ny*nz elements of the mesh type, x fastest;
 * `at_cathode` adds the image charge's potential.
 *  - SC_PREC_MIXED and SC_PREC_FP64 meshes with at most 128 nodes per axis:
 *    the hand-written pipeline in the mesh's precision, with its own cached
 *    potential Green spectrum (parity-reduced: even along every axis).  It
 *    uses the spare fourth lane of the mesh's packed field nodes as scratch
 *    (Ex, Ey, Ez are left as they are).
 *  - SC_PREC_PLAIN64 meshes and longer axes: the reference's schedule in
 *    FP64 with cuFFT. */
int sc_solve_potential(sc_mesh* mesh, int at_cathode, void* phi, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SPACECHARGE_GB300_H */
