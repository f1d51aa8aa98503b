/*
 * solvcon-gb300 C ABI: the drop-in boundary of the GPU CESE march.
 *
 * Plain C: opaque handles, plain pointers and sizes, integer status codes.
 * Every function returns SCG_OK (0) or one of the SCG_E* codes below, and the
 * message of the most recent failure on the calling thread is returned by
 * scg_last_error().  No C++ exception crosses this boundary.  Arrays are
 * exchanged in the reference's own layout: one contiguous row-major FP64 (or
 * int32) table per array, ghost rows first, so row i of a table with nghost
 * ghost rows is stored at (i + nghost) * row_width.
 *
 * Each declaration names the reference interface it replaces, by file:line
 * within solvcon's source tree.  A handle is not thread-safe: use one handle
 * from one thread at a time.
 */

#ifndef SCG_H
#define SCG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes (map onto the reference's exception types). */
#define SCG_OK 0
#define SCG_EINVAL 1   /* std::invalid_argument -> ValueError */
#define SCG_ERANGE 2   /* std::out_of_range -> IndexError */
#define SCG_ERUNTIME 3 /* std::runtime_error -> RuntimeError */
#define SCG_ECUDA 4    /* CUDA runtime failure -> RuntimeError */
#define SCG_ENOMEM 5   /* allocation failure -> MemoryError */

typedef struct scg_mesh scg_mesh;
typedef struct scg_euler scg_euler;
typedef struct scg_e1d scg_e1d;
typedef struct scg_st scg_st;

/* Message of the last failure on this thread ("" if none). */
const char * scg_last_error(void);
/* Number of CUDA kernels this library has launched in this process. */
int64_t scg_launch_count(void);
/* Number of device allocations (cudaMalloc) this library has made in this
 * process for its solver objects and per-call scratch (the device mesh
 * builder's Thrust buffers are not counted). */
int64_t scg_device_alloc_count(void);
/* Library version string. */
const char * scg_version(void);

/* ------------------------------------------------------------------------
 * Unstructured mesh, host side.
 * Replaces solvcon::StaticMesh (cpp/solvcon/mesh/StaticMesh.hpp:264-456) as
 * bound to Python by cpp/solvcon/mesh/pymod/wrap_StaticMesh.cpp:61-181.
 * ---------------------------------------------------------------------- */

/* Mesh array ids for scg_mesh_array. */
#define SCG_MESH_NDCRD 0
#define SCG_MESH_FCCND 1
#define SCG_MESH_FCNML 2
#define SCG_MESH_FCARA 3
#define SCG_MESH_CLCND 4
#define SCG_MESH_CLVOL 5
#define SCG_MESH_FCTPN 6
#define SCG_MESH_CLTPN 7
#define SCG_MESH_CLGRP 8
#define SCG_MESH_FCNDS 9
#define SCG_MESH_FCCLS 10
#define SCG_MESH_CLNDS 11
#define SCG_MESH_CLFCS 12
#define SCG_MESH_EDNDS 13
#define SCG_MESH_BNDFCS 14

/* StaticMesh(ndim, nnode, nface, ncell): StaticMesh.hpp:290-311. */
int scg_mesh_create(int ndim, int64_t nnode, int64_t nface, int64_t ncell, scg_mesh ** out);
int scg_mesh_destroy(scg_mesh * mesh);
/* A mesh built by other code -- the reference's own StaticMesh after
 * build_interior, build_boundary and build_ghost (its Gmsh reader's, a
 * pilot driver's), or anything producing the same tables -- taken over
 * verbatim, nothing rebuilt.  sizes[9] = ndim nnode nface ncell nbound
 * ngstnode ngstface ngstcell nedge (the size properties,
 * wrap_StaticMesh.cpp:97-106); tables[15] = the whole buffers, ghost rows
 * first, in SCG_MESH_* order, in the layout of the reference's table
 * properties (StaticMesh.hpp:434-451; float64 for ndcrd..clvol, int32 for
 * fctpn..bndfcs); a table with no rows may be null.  The tables are copied;
 * the core built on the mesh checks the connectivity on the device before
 * any kernel indexes through it. */
int scg_mesh_from_tables(const int64_t * sizes, const void * const * tables, scg_mesh ** out);
/* Append a boundary group with its facn table [nbound][3] verbatim (the
 * reference's StaticMeshBC name and facn, StaticMesh.hpp:159-251), for a mesh
 * taken over with scg_mesh_from_tables. */
int scg_mesh_adopt_bc(scg_mesh * mesh, const char * name, const int32_t * facn, int64_t nbound);
/* out[10] = ndim nnode nface ncell nbound ngstnode ngstface ngstcell nedge nbcs
 * (wrap_StaticMesh.cpp:97-106). */
int scg_mesh_sizes(const scg_mesh * mesh, int64_t * out);
/* Pointer to the live host table of one mesh array (valid until the next
 * build call); *dtype is 0 for float64 and 1 for int32; shape has up to 2
 * extents and nghost is the first-axis ghost count (StaticMesh.hpp:434-451). */
int scg_mesh_array(scg_mesh * mesh, int which, void ** data, int64_t * shape, int * nd, int64_t * nghost,
                   int * dtype);
/* build_interior(do_metric, do_edge): StaticMesh.hpp:363-374. */
int scg_mesh_build_interior(scg_mesh * mesh, int do_metric, int do_edge);
/* build_edge: StaticMesh_interior.cpp:566-621. */
int scg_mesh_build_edge(scg_mesh * mesh);
/* build_interior on the GPU: face extraction, de-duplication and numbering,
 * face-cell relations and metrics in device kernels, the tables copied back;
 * every table equals scg_mesh_build_interior's entry for entry
 * (StaticMesh_interior.cpp:17-977 restated per face and per cell).  Needs a
 * GPU and a mesh without ghost layer whose cells all have the mesh's
 * dimension (others go to the host builder or give SCG_EINVAL). */
int scg_mesh_build_interior_device(scg_mesh * mesh, int do_metric, int do_edge);
/* Number of CUDA devices visible (0 without a driver or a GPU). */
int scg_device_count(int * out);
/* add_bc(name, faces): StaticMesh_boundary.cpp:68-78. */
int scg_mesh_add_bc(scg_mesh * mesh, const char * name, const int32_t * faces, int64_t nface);
/* Name and facn table [nbound][3] of boundary group ibc (StaticMesh.hpp:159-251);
 * name is copied into buf of length buflen; facn may be null to query nbound. */
int scg_mesh_bc(const scg_mesh * mesh, int64_t ibc, char * buf, int64_t buflen, int32_t * facn, int64_t * nbound);
/* build_boundary: StaticMesh_boundary.cpp:103-182. */
int scg_mesh_build_boundary(scg_mesh * mesh);
/* build_ghost: StaticMesh_boundary.cpp:185-240. */
int scg_mesh_build_ghost(scg_mesh * mesh);
/* A mesh read from a Gmsh MSH 2.2 ASCII file's contents (nbyte bytes at
 * data): inout::Gmsh(data).to_block() (cpp/solvcon/inout/gmsh.cpp:14-118,
 * gmsh.hpp:70-285).  The elements of the highest dimension become the cells,
 * every node is kept, and the mesh comes back with build_interior,
 * build_boundary and build_ghost done.  A malformed file (wrong version,
 * missing or out-of-order sections) gives SCG_EINVAL; a node id out of range
 * SCG_ERANGE.  Free with scg_mesh_destroy. */
int scg_mesh_from_gmsh(const char * data, int64_t nbyte, scg_mesh ** out);
/* A mesh of hexahedra read from a Plot3D multi-block ASCII grid file's
 * contents: inout::Plot3d(data).to_block() (cpp/solvcon/inout/plot3d.cpp:
 * 14-155).  One hexahedron per grid cell of every block, blocks share no
 * nodes, and the mesh comes back with build_interior, build_boundary and
 * build_ghost done.  A malformed file gives SCG_EINVAL.  Free with
 * scg_mesh_destroy. */
int scg_mesh_from_plot3d(const char * data, int64_t nbyte, scg_mesh ** out);

/* ------------------------------------------------------------------------
 * Multi-dimensional Euler CESE core on the GPU.
 * Replaces solvcon::EulerCore (cpp/solvcon/multidim/euler.hpp:56-211) as bound
 * by cpp/solvcon/multidim/pymod/wrap_multidim.cpp:184-414.
 * ---------------------------------------------------------------------- */

/* Precision of the march. */
#define SCG_FP64 0        /* the reference's FP64 arithmetic */
/* The FP32 form of the EulerCore: FP32 state and flux arithmetic with
 * compensated face sums, mesh geometry kept in FP64 tables, FP64 totals and
 * CFL reduction.  The march rounds the FP64 geometry to FP32 where it uses
 * it; a mesh whose geometry (at this time increment) reaches 2^128 in
 * magnitude, or holds infinities or NaN, is refused with SCG_EINVAL when the
 * core is created or one of its CE geometry arrays is set. */
#define SCG_FP32_GEOM64 1
/* A faster EulerCore variant beside it: the same FP32 march with its
 * geometry (computed in FP64) stored in FP32, ~35% less traffic per cell. */
#define SCG_FP32_GEOM32 2
/* Euler1DCore's FP32 state (its coordinates stay FP64), and the FP32 pipe of
 * scg_fma_peak; as an EulerCore precision the same code as SCG_FP32_GEOM32. */
#define SCG_FP32 2

/* EulerCore array ids (wrap_multidim.cpp:381-408). */
#define SCG_EA_CEVOL 0
#define SCG_EA_CECND 1
#define SCG_EA_SFCND 2
#define SCG_EA_SFNML 3
#define SCG_EA_SO0C 4
#define SCG_EA_SO0N 5
#define SCG_EA_SO0T 6
#define SCG_EA_SO1C 7
#define SCG_EA_SO1N 8
#define SCG_EA_STM 9
#define SCG_EA_CFLO 10
#define SCG_EA_CFLC 11
#define SCG_EA_GAMMA 12

/* EulerCore operation ids for scg_euler_op (wrap_multidim.cpp:270-328). */
#define SCG_OP_PREPARE_CE 0
#define SCG_OP_UPDATE 1
#define SCG_OP_CALC_SOLT 2
#define SCG_OP_CALC_SOLN 3
#define SCG_OP_BC_SOLN 4
#define SCG_OP_CALC_CFL 5
#define SCG_OP_CALC_DSOLN 6
#define SCG_OP_BC_DSOLN 7
#define SCG_OP_MARCH_SUBSTEP 8
/* Not a reference operation: the solution state back to that of a new core
 * (the mesh, geometry and boundary conditions kept), for reusing a core. */
#define SCG_OP_RESET_STATE 9

/* Boundary kinds (euler.hpp:26-31). */
#define SCG_BC_NONREFL 0
#define SCG_BC_SLIPWALL 1
#define SCG_BC_INLET 2

/* Parameter ids. */
#define SCG_PARAM_SIGMA0 0
#define SCG_PARAM_TAUMIN 1
#define SCG_PARAM_TAUSCALE 2
#define SCG_PARAM_TIME_INCREMENT 3 /* read-only */

/* EulerCore(mesh, time_increment): euler_ce.cpp:15-29 (builds CE geometry on
 * the device).  The mesh must have its ghost layer built; the core copies what
 * it needs, so the mesh may be destroyed afterwards. */
int scg_euler_create(const scg_mesh * mesh, double time_increment, int precision, scg_euler ** out);
int scg_euler_destroy(scg_euler * core);
/* out[5] = ndim ncell ngstcell neq precision (wrap_multidim.cpp:247-268). */
int scg_euler_info(const scg_euler * core, int64_t * out);
/* sigma0/taumin/tauscale properties and time_increment (wrap_multidim.cpp:313-316). */
int scg_euler_get_param(const scg_euler * core, int which, double * value);
int scg_euler_set_param(scg_euler * core, int which, double value);
/* Shape (up to 3 extents) and ghost count of an array in the reference layout. */
int scg_euler_array_shape(const scg_euler * core, int which, int64_t * shape, int * nd, int64_t * nghost);
/* Copy a whole array (ghost rows first) device -> host / host -> device;
 * count is the number of float64 elements in the host buffer. */
int scg_euler_get(scg_euler * core, int which, double * host, int64_t count);
int scg_euler_set(scg_euler * core, int which, const double * host, int64_t count);
/* init_solution(gamma, rho, v, p): euler_solution.cpp:54-99. */
int scg_euler_init_solution(scg_euler * core, double gamma, double rho, const double * v, int nv, double p);
/* add_nonrefl/add_slipwall/add_inlet: euler_bc.cpp:324-391. */
int scg_euler_add_bc(scg_euler * core, int kind, const int32_t * faces, int64_t nface, const double * value,
                     int64_t nvalue);
/* clear_bc: euler.hpp:152. */
int scg_euler_clear_bc(scg_euler * core);
/* get_normal_matrix(ifc) -> out[ndim*ndim]: euler_bc.cpp:393-425. */
int scg_euler_normal_matrix(const scg_euler * core, int32_t ifc, double * out);
/* prepare_ce, update, calc_solt, calc_soln, bc_soln, calc_cfl, calc_dsoln,
 * bc_dsoln, march_substep: euler_march.cpp:307-348 and friends.  Synchronous. */
int scg_euler_op(scg_euler * core, int op);
/* march(steps): euler_march.cpp:350-359.  Asynchronous on the core's stream;
 * scg_euler_sync waits for it. */
int scg_euler_march(scg_euler * core, int64_t steps);
/* Not in the reference: scg_euler_set(SCG_EA_SO0N, so0n, n0),
 * scg_euler_set(SCG_EA_SO1N, so1n, n1) and scg_euler_march(steps) in one call
 * (the reference's array setters, wrap_multidim.cpp:381-408, then
 * march).  When both tables are whole-array ranges of scg_host_alloc blocks
 * the upload runs on a second stream in row chunks while the first substep
 * marches the cells whose rows are already up; otherwise the tables are set
 * as scg_euler_set does.  The state it leaves, and what a registered
 * delivery receives, equal set + march bit for bit.  Asynchronous like
 * scg_euler_march: the host tables must stay unchanged until scg_euler_sync
 * returns. */
int scg_euler_march_from_host(scg_euler * core, const double * so0n, int64_t n0, const double * so1n,
                              int64_t n1, int64_t steps);
int scg_euler_sync(scg_euler * core);
/* Not in the reference: have every later march also leave array `which`
 * (SCG_EA_SO0N or SCG_EA_SO1N, the whole array of `count` doubles in the
 * layout scg_euler_get gives) in the host block `host`.  An FP64 core's last
 * substep kernel writes the rows as it computes them, so the result crosses
 * the host link while the FP64-bound march runs instead of in a copy after
 * it; an FP32 core (latency-bound, its scattered row stores would not fill
 * whole lines) queues a coalesced gather into the block right after the
 * march.  After scg_euler_sync (or
 * any synchronous call) the block holds what scg_euler_get would return.
 * host must be a 16-byte aligned range of one scg_host_alloc block; NULL
 * stops the delivery.  A block freed while registered is dropped at the next
 * march and never written; free a block only after scg_euler_sync, since an
 * asynchronous march may still be writing it.  Batched marches
 * (scg_batch_march) do not deliver: they refuse a core with a registered
 * block (SCG_EINVAL) rather than leave it stale.  The replacement for the reference's pattern of
 * march(steps) followed by reading so0n / so1n (euler_march.cpp:350-359;
 * the so0n / so1n properties, multidim/pymod/wrap_multidim.cpp:393-396)
 * when the host reads every step. */
int scg_euler_deliver(scg_euler * core, int which, double * host, int64_t count);
/* Run the core on a caller-owned cudaStream_t (null restores its own). */
int scg_euler_set_stream(scg_euler * core, void * cuda_stream);
/* W-3/4 limiter firing bits of the last calc_dsoln per body cell: bit i set
 * when sigma_max of equation i was capped below sigma0/|cfl|
 * (euler_gradient.cpp:102-108).  out has ncell bytes. */
int scg_euler_limiter_mask(scg_euler * core, uint8_t * out);
/* FP64 totals sum_i so0n[i, :] * clvol[i] over body cells (out[neq]); the
 * mass/momentum/energy integrals of solvcon's EulerField
 * (solvcon/multidim/euler/_field.py:16-148). */
int scg_euler_totals(scg_euler * core, double * out);
/* The same totals without allocating any memory.  No counterpart in the
 * reference: it exists for callers that reserved their device memory up front
 * and must not allocate afterwards (a serving loop polling the totals of every
 * resident solve under a fixed HBM budget), because scg_euler_totals
 * allocates a per-call buffer with cudaMalloc and frees it with cudaFree, and
 * cudaFree synchronises the whole device.  Its partial sums live in a fixed
 * 131,136-byte device array (held by every GPU that loads the library until
 * exit) shared by all calls: at most 67,108,864 body cells (larger meshes
 * are rejected with SCG_EINVAL), the first call on a device looks up the
 * array's address, and calls that overlap on the GPU race -- issue them one
 * after the other.  Every call is synchronous: it copies the totals to the
 * host and waits for the core's stream, so it must not be made while that
 * stream is being captured into a CUDA graph. */
int scg_euler_totals_noalloc(scg_euler * core, double * out);
/* min and max of cflo over body cells (EulerField.calc_cfl_range). */
int scg_euler_cfl_range(scg_euler * core, double * out);
/* One scalar field of the newest solution (so0n) over the body cells, derived
 * on the device in FP64 and copied to out[ncell]; replaces the properties of
 * EulerField (solvcon/multidim/euler/_field.py:59-125), which derive the same
 * fields on the host from a full copy of so0n.  which: SCG_FIELD_* below;
 * SCG_FIELD_VELZ only in 3D, anything else SCG_EINVAL. */
#define SCG_FIELD_DENSITY 0
#define SCG_FIELD_VELX 1
#define SCG_FIELD_VELY 2
#define SCG_FIELD_VELZ 3
#define SCG_FIELD_SPEED 4
#define SCG_FIELD_PRESSURE 5
#define SCG_FIELD_MACH 6
#define SCG_FIELD_TOTAL_ENERGY 7
#define SCG_FIELD_CFL 8
int scg_euler_field(scg_euler * core, int which, double * out);
/* Device memory held by the core, in bytes. */
int scg_euler_device_bytes(const scg_euler * core, int64_t * out);

/* The core's CUDA stream (cudaStream_t) for stream-ordered event timing. */
int scg_euler_stream(const scg_euler * core, void ** out);
/* Per-launch CUDA-event timing of the fused march kernel: enable (resets the
 * record) or disable; stats return the summed duration and launch count. */
int scg_euler_profile(scg_euler * core, int on);
int scg_euler_profile_stats(scg_euler * core, double * ms_total, int64_t * launches);

/* ------------------------------------------------------------------------
 * 1D Euler CESE core on the GPU.
 * Replaces solvcon::onedim::Euler1DCore (cpp/solvcon/onedim/Euler1DCore.hpp:39-349)
 * as bound by cpp/solvcon/onedim/pymod/wrap_onedim.cpp:18-162.
 * ---------------------------------------------------------------------- */

/* Array ids: 0 coord [ncoord], 1 cfl [ncoord], 2 so0 [ncoord][3],
 * 3 so1 [ncoord][3], 4 gamma [ncoord]. */
#define SCG_E1D_COORD 0
#define SCG_E1D_CFL 1
#define SCG_E1D_SO0 2
#define SCG_E1D_SO1 3
#define SCG_E1D_GAMMA 4

/* Operation ids for scg_e1d_op (Euler1DCore.hpp:119-137, Euler1DCore.cpp:70-172). */
#define SCG_E1D_UPDATE_CFL 0
#define SCG_E1D_MARCH_HALF_SO0 1
#define SCG_E1D_MARCH_HALF_SO1 2
#define SCG_E1D_TREAT_BOUNDARY_SO0 3
#define SCG_E1D_TREAT_BOUNDARY_SO1 4
#define SCG_E1D_SETUP_MARCH 5
#define SCG_E1D_MARCH_HALF1 6
#define SCG_E1D_MARCH_HALF2 7

/* Euler1DCore(ncoord, time_increment): Euler1DCore.hpp:71-75, Euler1DCore.cpp:22-35. */
int scg_e1d_create(int64_t ncoord, double time_increment, scg_e1d ** out);
/* The same with the state precision: SCG_FP64 (the reference's arithmetic)
 * or SCG_FP32 (FP32 state, cfl and gamma; coordinates kept FP64, the spacing
 * between them formed in FP64 and rounded once to FP32).  Not in the
 * reference. */
int scg_e1d_create_precision(int64_t ncoord, double time_increment, int precision, scg_e1d ** out);
int scg_e1d_precision(const scg_e1d * h, int * precision);
int scg_e1d_destroy(scg_e1d * core);
/* clone(): Euler1DCore.hpp:58-62. */
int scg_e1d_clone(scg_e1d * core, scg_e1d ** out);
/* ncoord and time_increment (wrap_onedim.cpp:53-54). */
int scg_e1d_info(const scg_e1d * core, int64_t * ncoord, double * time_increment);
/* Whole-array copies device -> host / host -> device (wrap_onedim.cpp:83-104). */
int scg_e1d_get(scg_e1d * core, int which, double * host, int64_t count);
int scg_e1d_set(scg_e1d * core, int which, const double * host, int64_t count);
/* update_cfl, march_half_so0, march_half_so1_alpha<alpha>, treat_boundary_so0/so1,
 * setup_march, march_half1_alpha<alpha>, march_half2_alpha<alpha>
 * (wrap_onedim.cpp:107-150).  Synchronous. */
int scg_e1d_op(scg_e1d * core, int op, int odd_plane, int alpha);
/* march_alpha<alpha>(steps): Euler1DCore.hpp:339-349.  Asynchronous. */
int scg_e1d_march(scg_e1d * core, int alpha, int64_t steps);
int scg_e1d_sync(scg_e1d * core);
int scg_e1d_stream(const scg_e1d * core, void ** out);

/* ------------------------------------------------------------------------
 * Batched march of many independent Euler cores.  No single reference
 * counterpart: it runs EulerCore::march (euler_march.cpp:350-359) of many
 * cores at once, one launch per substep over a (core, row tile) work list,
 * replayed from a CUDA graph.  The cores must share ndim and precision, must
 * outlive the batch, and must not be used by other calls while a batch march
 * runs.
 * ---------------------------------------------------------------------- */

typedef struct scg_batch scg_batch;

/* block: 64, 128 or 256 threads per tile; persistent: grid sized to the
 * resident capacity (blocks stride over tiles) instead of one block per tile. */
int scg_batch_create(scg_euler * const * cores, int64_t ncore, int block, int persistent, scg_batch ** out);
int scg_batch_destroy(scg_batch * batch);
/* Point an existing batch at another set of cores (its stream, device tables
 * and occupancy are kept; the step graph is captured again at the next
 * march).  *done = 0, and nothing changes, when the new set needs another
 * kernel (other ndim, precision, or cell-type specialisation): create a new
 * batch then. */
int scg_batch_retarget(scg_batch * batch, scg_euler * const * cores, int64_t ncore, int * done);
/* out[5] = ncore, total body cells, tiles, grid, block. */
int scg_batch_info(const scg_batch * batch, int64_t * out);
/* march(steps) of every core; synchronous.  SCG_EINVAL, and nothing
 * marched, when a core has host blocks registered with scg_euler_deliver
 * (a batched march does not write them). */
int scg_batch_march(scg_batch * batch, int64_t steps);
/* Device time of the last scg_batch_march's kernels (CUDA events, ms). */
int scg_batch_last_ms(const scg_batch * batch, double * ms);
int scg_batch_stream(const scg_batch * batch, void ** out);

/* ------------------------------------------------------------------------
 * 1D spacetime scalar CESE solvers on the GPU (periodic boundary, one variable).
 * Replaces solvcon::spacetime::LinearScalarSolver / InviscidBurgersSolver
 * (cpp/solvcon/spacetime/kernel/linear_scalar.hpp:27-87,
 * kernel/inviscid_burgers.hpp:30-109) and their SolverBase march
 * (cpp/solvcon/spacetime/core.hpp:946-1036).
 * ---------------------------------------------------------------------- */

#define SCG_ST_LINEAR_SCALAR 0
#define SCG_ST_INVISCID_BURGERS 1
/* Array ids: 0 xcoord, 1 so0, 2 so1, 3 cfl, each [2 * ncelm + 5]. */
#define SCG_ST_X 0
#define SCG_ST_SO0 1
#define SCG_ST_SO1 2
#define SCG_ST_CFL 3

/* Solver(grid, time_increment): xcoord is the grid's coordinate table
 * (Grid::xcoord, core.cpp:52-99) of 2 * ncelm + 5 entries. */
int scg_st_create(int kind, const double * xcoord, int64_t ncelm, double time_increment, scg_st ** out);
int scg_st_destroy(scg_st * solver);
/* set_time_increment (core.hpp:836). */
int scg_st_set_time_increment(scg_st * solver, double time_increment);
int scg_st_get(scg_st * solver, int which, double * host, int64_t count);
int scg_st_set(scg_st * solver, int which, const double * host, int64_t count);
/* op ids as for scg_e1d_op: 0 update_cfl, 1 march_half_so0, 2 march_half_so1_alpha,
 * 3/4 treat_boundary_so0/so1, 5 setup_march, 6 march_half1_alpha,
 * 7 march_half2_alpha (core.hpp:946-1025).  Synchronous. */
int scg_st_op(scg_st * solver, int op, int odd_plane, int alpha);
/* march_alpha<alpha>(steps): core.hpp:1027-1036.  Asynchronous. */
int scg_st_march(scg_st * solver, int alpha, int64_t steps);
int scg_st_sync(scg_st * solver);
/* The solver's CUDA stream (cudaStream_t), for stream-ordered event timing
 * (no reference counterpart: measurement plumbing). */
int scg_st_stream(const scg_st * solver, void ** out);

/* ------------------------------------------------------------------------
 * Timing and host-memory helpers (no reference counterpart: measurement
 * plumbing of this library).
 * ---------------------------------------------------------------------- */

/* Not in the reference: round n FP64 values to FP32 on the device exactly as
 * the FP32 march rounds its FP64 geometry tables where it uses them
 * (round to nearest even, formed on the integer pipe; values below FP32's
 * normal range give a signed zero, and values of magnitude 2^128 and beyond,
 * which a core refuses, are not defined here), for checking that rounding.  Synchronous; allocates its own device buffers. */
int scg_geometry_round(const double * in, float * out, int64_t n);
/* Not in the reference: n FP64 quotients x[i] / d[i] on the device, q by
 * the spacetime march's division from a tabulated reciprocal (Markstein's
 * method) and qdiv by the IEEE division, for checking that the two agree bit
 * for bit; rcp[i] is the multi-dimensional FP64 march's reciprocal of d[i]
 * (Newton's iteration, within one ulp of 1 / d).  Synchronous; allocates its
 * own device buffers. */
int scg_divide_check(const double * x, const double * d, double * q, double * qdiv, double * rcp, int64_t n);
/* Device FMA throughput in TFLOP/s for SCG_FP64 or SCG_FP32 (a register-only
 * FMA chain over all SMs, iters FMAs-per-accumulator). */
int scg_fma_peak(int precision, int iters, double * tflops);
/* Page-locked host blocks, mapped into the device's address space.  A table
 * that lies inside such a block moves through scg_euler_get / scg_euler_set
 * with one gather or scatter kernel over the host link and no staging copy;
 * any other host pointer goes through a device staging table. */
int scg_host_alloc(int64_t nbytes, void ** out);
int scg_host_free(void * ptr);
/* CUDA events (cudaEvent_t) recorded on a stream, and their elapsed time. */
int scg_event_create(void ** out);
int scg_event_destroy(void * ev);
int scg_event_record(void * ev, void * stream);
int scg_event_elapsed(void * ev0, void * ev1, double * ms);
int scg_device_sync(void);

#ifdef __cplusplus
}
#endif

#endif /* SCG_H */
