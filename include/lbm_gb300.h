/*
 * lbm_gb300.h -- C ABI of the GB300 (sm_103a) D2Q9 BGK lattice Boltzmann hot path.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, launches
 * asynchronously on the caller's CUDA stream (`stream` is a cudaStream_t
 * passed as void*, NULL = legacy default stream), allocates nothing, and
 * returns 0 on success or a negative LBM_ERR_* code; lbm_last_error() then
 * holds a one-line message for the calling thread.
 *
 * Reference-facing layout (the arrays the reference's NumPy functions take,
 * C order): f[nx][ny][9], rho[nx][ny], u[nx][ny][2], all float64, x = axis 0.
 * D2Q9 directions: c = (0,0),(1,0),(0,1),(-1,0),(0,-1),(1,1),(-1,1),(-1,-1),(1,-1)
 * (src/lattice_boltzmann_method.py:14-26).
 *
 * Resident layout (the hot loop): structure-of-arrays population planes
 * pop[9][ny][pitch] with x contiguous; the state kept between steps is the
 * post-collision, pre-streaming population (see lbm_lattice_*).
 */
#ifndef LBM_GB300_H
#define LBM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define LBM_OK 0
#define LBM_ERR_ARG (-1)      /* shape/pointer/argument check failed (reference: AssertionError) */
#define LBM_ERR_OMEGA (-2)    /* omega outside (0, 2): lattice_boltzmann_method.py:212 */
#define LBM_ERR_CUDA (-3)     /* a CUDA runtime call failed */
#define LBM_ERR_UNSUPPORTED (-4)

/* ---- per-node boundary sources ------------------------------------------ */
/* For every node and direction i the post-streaming population comes from one source:
 *   PULL   : periodic streaming, f_pre(x - c_i, i)             (np.roll, lattice_boltzmann_method.py:156-157)
 *   BOUNCE : f_pre(x, opp(i)) - kconst[kset][i]               (rigid_wall :108-109, moving_wall :207-210,
 *                                                              rigid_object :153-163, boundary_utils.py:179-201)
 *   CONST  : cconst[cset][i]                                  (inlet :250-251)
 *   OUTLET : f_prev(x - 1, i), only at column nx-1            (outlet :279-280)
 * desc bits 2i..2i+1 hold the source of direction i, bits 18..21 kset, 22..25 cset. */
#define LBM_SRC_PULL 0u
#define LBM_SRC_BOUNCE 1u
#define LBM_SRC_CONST 2u
#define LBM_SRC_OUTLET 3u
#define LBM_DESC_KSET_SHIFT 18
#define LBM_DESC_CSET_SHIFT 22
#define LBM_MAX_SETS 16

typedef struct lbm_geometry {
  int32_t nx, ny;
  /* device, [ny][(nx+31)/32] words: bit (x%32) of word x/32 marks a node whose
   * descriptor is not all-PULL; NULL means every node streams periodically. */
  const uint32_t* bcmask;
  /* device, [ny][nx] descriptors (read only where bcmask has the bit set). */
  const uint32_t* desc;
  int32_t n_kset, n_cset;
  double kconst[LBM_MAX_SETS][9]; /* moving-wall terms 2 w_i rho_avg c_i.u_w / c_s^2 (0 = rigid) */
  double cconst[LBM_MAX_SETS][9]; /* fixed populations (inlet equilibrium) */
  /* periodic_with_pressure_variations (boundary_conditions.py:286-348): before
   * streaming, column 0 / column nx-1 directions in pressure_in_dirs /
   * pressure_out_dirs (bit masks) are rewritten from columns nx-2 / 1. */
  int32_t pressure;
  uint32_t pressure_in_dirs, pressure_out_dirs;
  double rho_in, rho_out;
  int32_t outlet; /* some node uses LBM_SRC_OUTLET */
  /* device, the n_bcnodes linear indices y*nx + x (ascending) of the nodes with a
   * bcmask bit.  With it, on lattices of at least 2^22 nodes in the 16-bit
   * storages and 2^25 in the others (or with LBM_FLAG_BC_SPLIT), the vectorised
   * step runs its boundary-free body over the whole lattice and then recomputes
   * just these nodes with their sources; NULL, a smaller lattice or
   * LBM_FLAG_BC_INLINE applies the sources inside the step. */
  const int32_t* bcnodes;
  int32_t n_bcnodes;
  /* Plain inlet and outlet columns (all zero: none).  edge_inlet_desc is the
   * descriptor of the nodes of column 0 that take only the inlet populations
   * (all nine directions CONST from one constant set), edge_outlet_desc that
   * of the nodes of column nx-1 that take only directions 3, 6, 7 from the
   * outlet memory (the others stream); each is set only when every node of
   * its column has a descriptor.  The last n_bcnodes_edge entries of bcnodes
   * are the nodes with these two descriptors (the others come first).  The
   * batched step applies them inside its boundary-free launch, where they cost
   * no scattered column accesses, and passes over the other entries only. */
  uint32_t edge_inlet_desc, edge_outlet_desc;
  int32_t n_bcnodes_edge;
  /* Reference velocity of the reference-shifted 16-bit storages
   * (LBM_STORE_F16R, LBM_STORE_BF16R): they keep f_i - c_i with c_i the
   * equilibrium at rho = 1 and this velocity; every call on one resident state
   * must give the same value.  The other storages do not use it (leave it 0);
   * every call checks that it lies inside (-0.5, 0.5). */
  double dev_ref_ux, dev_ref_uy;
} lbm_geometry;

/* ---- storage / arithmetic of the resident state ------------------------- */
#define LBM_STORE_F64 0   /* 72 B per node, the drop-in */
#define LBM_STORE_F32 1   /* 36 B per node */
#define LBM_STORE_F16S 2  /* 18 B per node, 1024 (f_i - w_i) in binary16 */
#define LBM_STORE_BF16S 3 /* 18 B per node, f_i - w_i in bfloat16 */
#define LBM_STORE_FX64 4  /* 72 B per node, round((f_i - w_i) 2^56) in int64: float64 accuracy, no float64 arithmetic */
/* The reference-shifted 16-bit storages: as F16S / BF16S with w_i replaced by
 * c_i, the equilibrium at rho = 1 and the geometry's (dev_ref_ux, dev_ref_uy).
 * A flow near a uniform velocity (a channel at its inlet velocity) then keeps
 * smaller stored deviations and smaller rounding errors.  The vectorised
 * kernels run them at 4 nodes per thread (the LBM_FLAG_NPT field is ignored)
 * and the batched step at npt 2 or 4 and 128 threads. */
#define LBM_STORE_F16R 5  /* 18 B per node, 1024 (f_i - c_i) in binary16 */
#define LBM_STORE_BF16R 6 /* 18 B per node, f_i - c_i in bfloat16 */

#define LBM_FLAG_EXACT 1  /* float64 arithmetic in the reference's NumPy operation order, no FMA contraction */
#define LBM_FLAG_GENERIC 2 /* use the one-node-per-thread kernel instead of the vectorised one */
#define LBM_FLAG_NPT_SHIFT 4 /* bits 4..7: nodes per thread of the vectorised kernel (0 = default) */
#define LBM_FLAG_STOCHASTIC 256 /* 16-bit storages: round stored deviations stochastically */
#define LBM_FLAG_BC_INLINE 1024 /* boundary sources inside the vectorised step even when g->bcnodes is set */
#define LBM_FLAG_BC_SPLIT 2048  /* the boundary-node pass even below the size from which it is taken by default */

/* ---- library ------------------------------------------------------------ */
int lbm_version(void);
const char* lbm_last_error(void);
/* Number of your kernels launched by this thread since the last reset. */
int64_t lbm_launch_count(int reset);

/* ---- component operators, reference layout, float64 ------------------------ */
/* compute_density, lattice_boltzmann_method.py:93-105. rho[n] = sum_i f[n][i]. */
int lbm_density_f64(const double* f, double* rho, int64_t n_nodes, void* stream);
/* compute_velocity_field, lattice_boltzmann_method.py:108-137 (u = 0 where rho == 0). */
int lbm_velocity_f64(const double* rho, const double* f, double* u, int64_t n_nodes, void* stream);
/* equilibrium_distr_func, lattice_boltzmann_method.py:162-188 (any leading shape, flattened). */
int lbm_equilibrium_f64(const double* rho, const double* u, double* feq, int64_t n_nodes, void* stream);
/* streaming, lattice_boltzmann_method.py:140-159 (periodic, out of place). */
int lbm_streaming_f64(const double* f, double* f_out, int32_t nx, int32_t ny, void* stream);
/* the collision line of lattice_boltzmann_step, lattice_boltzmann_method.py:213-215. */
int lbm_collide_f64(const double* f, const double* rho, const double* u, double omega,
                    double* f_pre, int64_t n_nodes, int32_t flags, void* stream);
/* Applies the BOUNCE / CONST / OUTLET sources of `g` to f_post in place: the
 * boundary closures rigid_wall, moving_wall, rigid_object, inlet, outlet
 * (boundary_conditions.py:78-283) compiled into one descriptor. */
int lbm_apply_boundary_f64(const lbm_geometry* g, const double* f_pre, const double* f_prev,
                           double* f_post, void* stream);
/* periodic_with_pressure_variations' closure (boundary_conditions.py:320-346), in place on f_pre. */
int lbm_pressure_prestream_f64(const lbm_geometry* g, double* f_pre, const double* rho,
                               const double* u, void* stream);
/* The single-rank periodic ghost exchange of a ghost-padded (nx+2, ny+2, 9)
 * array (parallelization_utils.py:23-50 with every neighbour being this rank). */
int lbm_halo_fill_f64(double* f, int32_t nx_padded, int32_t ny_padded, void* stream);

/* ---- fused step, reference layout ------------------------------------------ */
/* lattice_boltzmann_step(f, rho, u, omega, boundary) (lattice_boltzmann_method.py:191-228)
 * with the boundary given as a compiled descriptor `g` (NULL bcmask = no boundary):
 * collision with the passed-in rho,u, pressure rewrite, streaming, boundary
 * sources and the moments, in two kernels.  `scratch` must hold
 * lbm_step_scratch_bytes(nx, ny) bytes (device). */
size_t lbm_step_scratch_bytes(int32_t nx, int32_t ny);
int lbm_step_f64(const lbm_geometry* g, const double* f, const double* rho, const double* u,
                 double omega, double* f_out, double* rho_out, double* u_out, void* scratch,
                 int32_t flags, void* stream);

/* The same step on HOST buffers in the reference layout (what the reference's
 * drivers hold: NumPy arrays; pinned memory lets the copies run asynchronously).
 * The lattice is cut into `slabs` ranges of x (0: one per 2^18 nodes, at most
 * 32), which are contiguous in the reference layout: slab k+1 is copied in
 * while slab k is collided and streamed and slab k-1 is copied out, on three
 * internal streams, so the two copy directions and the kernels overlap.  The
 * caller's `stream` waits for all of it.  `scratch` must hold
 * lbm_step_host_scratch_bytes(nx, ny) bytes (device).  Results are identical
 * to lbm_step_f64's. */
size_t lbm_step_host_scratch_bytes(int32_t nx, int32_t ny);
int lbm_step_f64_host(const lbm_geometry* g, const double* f, const double* rho, const double* u,
                      double omega, double* f_out, double* rho_out, double* u_out, void* scratch,
                      size_t scratch_bytes, int32_t flags, int32_t slabs, void* stream);

/* ---- fused step without allocation ------------------------------------------ */
/* No counterpart in the reference.  The same step as lbm_step_f64, for callers
 * that cannot allocate device memory: instead of a caller-provided `scratch`
 * it uses a static device array of LBM_NOALLOC_SCRATCH_BYTES compiled into the
 * library, which every GPU that loads the library holds until the process
 * exits.  A lattice needing more scratch than that, (9*pitch*ny + 3*ny)*8
 * bytes with pitch = nx rounded up to 32 (about 116 000 nodes), is rejected
 * with LBM_ERR_ARG.  The first call in each device context (per device, and
 * again after cudaDeviceReset) looks the array's address up with
 * cudaGetSymbolAddress, so make that first call before any stream capture.
 * Every call shares the array: calls that overlap on the GPU race. */
#define LBM_NOALLOC_SCRATCH_BYTES ((size_t)8 << 20)
int lbm_step_f64_noalloc(const lbm_geometry* g, const double* f, const double* rho, const double* u,
                         double omega, double* f_out, double* rho_out, double* u_out, int32_t flags,
                         void* stream);

/* ---- resident lattice (the hot loop) ----------------------------------------- */
/* State: pop[9][ny][pitch] (storage type per LBM_STORE_*) holding the
 * post-collision populations of the last step, plus aux[3][ny] (float64 for
 * F64 storage, float32 otherwise) holding the pre-collision populations 3,6,7
 * of column nx-2 that the outlet reads one step later.  pitch must be >= nx
 * and a multiple of 8. */
size_t lbm_lattice_pop_bytes(int32_t nx, int32_t ny, int64_t pitch, int32_t storage);

/* First step of a run: collide the reference-layout state (f, and rho,u when
 * given, else their moments) into pop_out/aux_out. */
int lbm_lattice_init(const lbm_geometry* g, int32_t storage, const double* f, const double* rho,
                     const double* u, double omega, void* pop_out, int64_t pitch, void* aux_out,
                     int32_t flags, void* stream);
/* nsteps fused pull-stream + boundary + collide steps, ping-ponging between
 * (pop_a, aux_a) and (pop_b, aux_b), starting from pop_a.  After an odd
 * number of steps the state is in pop_b.  When rho_out/u_out are not NULL
 * the moments of the pre-collision state of the LAST step are written as
 * SoA planes rho[ny][pitch], u[2][ny][pitch] (float64).  With LBM_FLAG_STOCHASTIC
 * the 16-bit storages round their stored deviations stochastically; step s of
 * the call draws its random bits from (seed, s, node, direction). */
int lbm_lattice_run(const lbm_geometry* g, int32_t storage, void* pop_a, void* pop_b, int64_t pitch,
                    void* aux_a, void* aux_b, double omega, int32_t nsteps, double* rho_out,
                    double* u_out, int32_t flags, uint32_t seed, void* stream);
/* Options of lbm_lattice_run_opts (any field may be zero / NULL).
 *   step_counter : device int.  When set, step s of the call draws its random
 *                  bits from (seed + s + *step_counter) read on the device, and
 *                  a last kernel adds nsteps to *step_counter.  A captured CUDA
 *                  graph of the call then draws new bits on every replay
 *                  (the counter holds the step index), where a seed passed by
 *                  value would repeat them.  Without it, step s uses (seed + s).
 *   probe_*      : the fused step appends (ux, uy) of node (probe_x, probe_y),
 *                  the velocity of the post-streaming state it collides, at
 *                  probe_buf[2 * (*probe_count)++] while the count is below
 *                  probe_cap: the per-step probe of the reference's drivers
 *                  (np.linalg.norm(velocity[px, py]) each step, src/experiments.py:690,703-704)
 *                  without a host round trip.  A probe keeps the boundary sources
 *                  inside the step (no boundary-node pass), so the node is
 *                  recorded once per step. */
typedef struct lbm_run_options {
  int32_t* step_counter;
  int32_t probe_x, probe_y, probe_cap;
  double* probe_buf;
  int32_t* probe_count;
} lbm_run_options;
/* lbm_lattice_run with options; lbm_lattice_run(...) is lbm_lattice_run_opts(..., NULL, stream). */
int lbm_lattice_run_opts(const lbm_geometry* g, int32_t storage, void* pop_a, void* pop_b, int64_t pitch,
                         void* aux_a, void* aux_b, double omega, int32_t nsteps, double* rho_out,
                         double* u_out, int32_t flags, uint32_t seed, const lbm_run_options* opt,
                         void* stream);
/* Materialise the current (post-streaming, post-boundary) state in the
 * reference layout: f_out[nx][ny][9], rho_out[nx][ny], u_out[nx][ny][2]
 * (any may be NULL). */
int lbm_lattice_read(const lbm_geometry* g, int32_t storage, const void* pop, int64_t pitch,
                     const void* aux, double* f_out, double* rho_out, double* u_out, void* stream);

/* ---- exact global moments ---------------------------------------------------------- */
/* out[3] (device) = (sum rho, sum jx, sum jy) of a reference-layout f[n][9],
 * summed exactly in 128-bit fixed point (round(f 2^53)), so the result does not
 * depend on the order of the additions; NaN when some |f| >= 2.  Replaces the
 * host np.sum checks of the drivers and tests (e.g. tests/test_mass_preservation.py:20-33).
 * `scratch` holds lbm_reduce_scratch_bytes(n) bytes (device). */
size_t lbm_reduce_scratch_bytes(int64_t n_nodes);
int lbm_reduce_moments_f64(const double* f, int64_t n_nodes, void* scratch, size_t scratch_bytes, double* out,
                           void* stream);

/* ---- batched lattices ----------------------------------------------------------- */
/* Many lattices of different sizes, one storage type, advanced together: one
 * launch per time step covers every live lattice (a flat list of tiles of
 * consecutive node chunks walked by a grid), followed by the boundary-node
 * pass (lbm_batch_build).  Lattice j is live for global steps
 * [s0, s_end); at global step g it reads pop_a when (g - s0) is even.  The
 * global step is *gbase (device int) plus the launch's index, and
 * lbm_batch_run ends with a kernel adding nsteps to *gbase, so a captured
 * CUDA graph of one lbm_batch_run call can be replayed.  The probe, when
 * probe_buf is set, appends (ux, uy) of node (probe_x, probe_y) each step at
 * probe_buf[2 * (*probe_count)++] while the count is below probe_cap.
 * No reference counterpart as a whole: it runs many drivers' loops
 * (src/experiments.py:650-720) at once. */
typedef struct lbm_batch_lattice {
  const lbm_geometry* g;
  void* pop_a;
  void* pop_b;
  void* aux_a;
  void* aux_b;
  int64_t pitch;
  double omega;
  int32_t s0, s_end;
  int32_t probe_x, probe_y, probe_cap;
  double* probe_buf;
  int32_t* probe_count;
  uint32_t seed;  /* stochastic rounding: random bits from (seed, g - s0, node, direction) */
  int32_t flags;  /* LBM_FLAG_STOCHASTIC, LBM_FLAG_BC_INLINE, LBM_FLAG_BC_SPLIT */
  int32_t rows;   /* runs per tile (0 = 1): a tile is `rows` runs of `threads` consecutive chunks of `npt`
                   nodes, chunks numbered row by row (a run may cross a row end) */
} lbm_batch_lattice;

size_t lbm_batch_table_bytes(int32_t n);
/* Writes the device work table (table_bytes >= lbm_batch_table_bytes(n)) for
 * tiles of `rows` runs of `threads` threads x `npt` nodes; synchronises `stream`.
 * *bc_chunks receives the boundary-node plan that lbm_batch_run takes: -1 when
 * the boundary sources run inside the step (some lattice has boundary nodes
 * but no list of them or sets LBM_FLAG_BC_INLINE, or the lattices hold fewer
 * than 2^20 nodes in total and none sets LBM_FLAG_BC_SPLIT: a second launch
 * per step would double the fixed cost of a small batch), else the number of
 * 128-node chunks of pass nodes: each step is then a boundary-free launch over
 * every node followed by a boundary-node pass over the chunks (bit-identical
 * results, fewer registers in the hot kernel). */
int lbm_batch_build(const lbm_batch_lattice* lat, int32_t n, int32_t npt, int32_t threads, void* table,
                    size_t table_bytes, int32_t* total_tiles, int32_t* bc_chunks, void* stream);
/* nsteps batched steps with `blocks` persistent blocks (0 = fill the GPU; more
 * than half the tile count = one tile per block, a plain grid);
 * total_tiles and bc_chunks as lbm_batch_build returned them. */
int lbm_batch_run(const void* table, int32_t n, int32_t total_tiles, int32_t bc_chunks, int32_t storage,
                  int32_t npt, int32_t threads, int32_t* gbase, int32_t nsteps, int32_t blocks, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* LBM_GB300_H */
