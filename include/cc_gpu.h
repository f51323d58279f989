/*
 * cc_gpu.h - C ABI of the GB300 connected-components library (libccgpu.so).
 *
 * This is the drop-in boundary for the connected-components (CC) solve of
 * sebalamm/components.  The reference reaches that solve through a C++ class
 * API used by its five drivers:
 *
 *     X comp(const Config &conf, PEID rank, PEID size);
 *     comp.FindComponents(G, labels);
 *
 *   app/exp_contraction.cpp:104-105   ExponentialContraction
 *   app/all_reduce.cpp:97-98          AllReduce<StaticGraph>
 *   app/local_contraction.cpp:114,142 LocalContraction
 *   app/shortcuts.cpp:117,145         ShortcutPropagation
 *   app/labels.cpp:101                Propagation
 *
 * Here one call, cc_gpu_run(), replaces that pair.  The graph travels as a
 * symmetric CSR (the reference's StaticGraph layout, lib/data_structures/
 * static_graph.h:120-171, 423-437) and the labels come back canonical: every
 * vertex gets the minimum vertex id of its component.  The reference's own
 * labels are not canonical (exponential_contraction.h:872,887 labels
 * unresolved vertices n+gid), so both sides are compared after
 * canonicalisation.  The C++ class names are provided on top of this ABI by
 * include/components_gb300.hpp.
 *
 * Errors are returned as an int status; the library never calls exit().  The
 * reference has no status codes: it calls exit(1) or MPI_Finalize
 * (io_utils.h:53-55, dynamic_contraction.h:437-438, comm_utils.h:58-60).
 *
 * Threading: one context (cc_ctx) owns one CUDA stream and one device arena;
 * a context must not be used by two host threads at once.  cc_gpu_run() uses
 * a per-thread default context on the current CUDA device.
 */
#ifndef CC_GPU_H_
#define CC_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
enum {
  CC_OK = 0,
  CC_ERR_INVALID = 1,        /* bad argument, malformed CSR or config */
  CC_ERR_OOM = 2,            /* device or pinned host allocation failed */
  CC_ERR_CUDA = 3,           /* a CUDA runtime call failed */
  CC_ERR_NO_CONVERGENCE = 4, /* an iterative loop hit its round cap */
  CC_ERR_TIMEOUT = 5,        /* a bounded device-side wait gave up */
  CC_ERR_UNSUPPORTED = 6,    /* option combination not provided */
  CC_ERR_BUSY = 7            /* serving queue full / over the HBM budget */
};

/* where the caller's pointers live */
enum { CC_HOST = 0, CC_DEVICE = 1 };

/*
 * Symmetric CSR of an undirected graph.  Vertex ids are 0..n-1; every
 * undirected edge {u,w} appears as the two directed entries u->w and w->u
 * (reference: StaticGraph built from symmetric generator edge lists,
 * graph_io.h:68-160).  Self-loops are ignored.  num_parts is the number of
 * virtual ranks P: vertex v belongs to the contiguous range of rank r with
 * the reference's split  n/P + (r < n%P)  (graph_io.h:308-313).
 */
typedef struct cc_csr {
  uint64_t n;               /* number of vertices */
  uint64_t m_dir;           /* number of directed adjacency entries */
  const uint64_t *row_ptr;  /* n+1 offsets into col */
  const void *col;          /* m_dir neighbour ids, id_bytes each */
  uint32_t id_bytes;        /* 4 (uint32 ids) or 8 (uint64 ids) */
  uint32_t num_parts;       /* virtual ranks P >= 1 */
  uint32_t where;           /* CC_HOST or CC_DEVICE for row_ptr and col; device row_ptr
                               8-byte aligned and col aligned to id_bytes, else
                               CC_ERR_INVALID before any launch */
  uint32_t reserved;        /* must be 0 */
} cc_csr;

/* The five driver options of app/ (one solver class each). */
typedef enum cc_algo {
  CC_EXP = 0,       /* ExponentialContraction (exponential_contraction.h:40) */
  CC_LOCAL = 1,     /* LocalContraction       (local_contraction.h:39)       */
  CC_SHORTCUTS = 2, /* ShortcutPropagation    (shortcut_propagation.h:38)    */
  CC_LABELS = 3,    /* Propagation            (propagation.h:38)             */
  CC_ALLREDUCE = 4  /* AllReduce<G>           (all_reduce.h:34)              */
} cc_algo;

/*
 * Mirror of the solver-relevant fields of Config (lib/config.h:29-87) with the
 * defaults of ParseParameters (app/parse_parameters.h:30-100); fill it with
 * cc_config_default().  I/O and generator fields stay on the host side.
 */
typedef struct cc_config {
  double beta;                /* -beta      0.1  exponential shift rate      */
  uint32_t seq;               /* -seq       1    sequential limit factor     */
  uint32_t prop_iterations;   /* -pi        3    (accepted; unused upstream) */
  uint32_t number_of_hitters; /* -heavy-hitters 0 shortcut request filter    */
  uint32_t degree_threshold;  /* -hd-thres  16   hub threshold factor        */
  uint32_t degree_limit;      /* -deg       100                              */
  float hd_sf;                /* -hd-sf     0.5  neighbourhood sampling      */
  uint8_t fixed_seq;          /* -fixed-seq                                  */
  uint8_t contraction;        /* -contraction (two-level component graph)    */
  uint8_t direct;             /* -direct                                     */
  uint8_t single;             /* -single (one-level component graph)         */
  uint8_t bfs;                /* -bfs (start-time gated decomposition)       */
  uint8_t replicate;          /* -replicate (hub vertices)                   */
  uint8_t regular;            /* -regular   accepted and ignored             */
  uint8_t overalloc;          /* -overalloc accepted and ignored             */
  uint8_t verbose;            /* -verbose                                    */
  uint8_t pad_[3];
} cc_config;

#define CC_MAX_LEVELS 64
#define CC_MAX_KSTATS 32

/* Per-kernel timing (CUDA events on the context stream), filled when
   profiling is on (cc_ctx_set_profiling). */
typedef struct cc_kernel_stat {
  char name[32];
  uint32_t launches;
  uint32_t pad_;
  double ms;       /* summed device time of the launches */
  uint64_t bytes;  /* summed algorithmic bytes of the launches */
} cc_kernel_stat;

/* Statistics of the last solve on a context (cc_gpu_stats / cc_ctx_stats). */
typedef struct cc_stats {
  uint32_t levels;                          /* contraction levels executed   */
  uint32_t rounds_total;                    /* iterative rounds, all levels  */
  uint32_t rounds[CC_MAX_LEVELS];           /* rounds per level              */
  uint64_t level_vertices[CC_MAX_LEVELS];   /* vertices of each level graph  */
  uint64_t level_edges[CC_MAX_LEVELS];      /* directed edges of each level  */
  uint64_t bytes_algorithmic;               /* sum of algorithmic bytes      */
  uint64_t kernel_launches;                 /* kernels launched by the solve */
  uint64_t num_components;                  /* components incl. isolated     */
  uint64_t h2d_bytes, d2h_bytes;            /* copies made for HOST buffers  */
  double solve_ms;                          /* device time of the solve      */
  double total_ms;                          /* incl. host<->device copies    */
  /* driver compatibility: GetCommTime/GetSendVolume/GetReceiveVolume
     (exponential_contraction.h:325-335).  No exchange happens on one
     device, so they are always 0. */
  double comm_time;
  uint64_t send_volume, recv_volume;
  uint32_t nkernels;                        /* entries used in kernels[]     */
  uint32_t pad_;
  cc_kernel_stat kernels[CC_MAX_KSTATS];
} cc_stats;

typedef struct cc_ctx cc_ctx;

/* ---- single-graph solve -------------------------------------------------- */

/* Fill *cfg with the ParseParameters defaults (parse_parameters.h:35-75). */
void cc_config_default(cc_config *cfg);

/*
 * Solve CC of *g with the solver `algo` and write canonical labels (minimum
 * vertex id of the component, id_bytes wide) to labels_out.  labels_out lives
 * where g->where says (host or device).  seed is Config::seed.  Replaces
 * X(conf, rank, size).FindComponents(G, labels) for one rank per GPU.
 */
int cc_gpu_run(const cc_csr *g, cc_algo algo, const cc_config *cfg,
               uint64_t seed, void *labels_out);

/* Statistics of the last cc_gpu_run() of this thread. */
int cc_gpu_stats(cc_stats *out);

/* Text of a status code, or of the last error of this thread for CC_ERR_CUDA. */
const char *cc_gpu_strerror(int status);

/* Validate a CSR (sizes, monotone offsets, ids < n, symmetry when check_sym);
   runs on the host for CC_HOST graphs and on the device for CC_DEVICE. */
int cc_csr_validate(const cc_csr *g, int check_sym);

/*
 * Allocation-free solve, for callers that cannot allocate device memory when
 * they solve: a plugin's enqueue() in an inference runtime, a process whose
 * device memory is pre-reserved by its own allocator, or a latency-critical
 * loop that cannot take the device synchronisation of cudaMalloc/cudaFree.
 * No counterpart in the reference.  Same labels as cc_gpu_run(CC_ALLREDUCE)
 * (and CC_EXP with one rank): labels_out[v] = minimum vertex id of v's
 * component.  All pointers are device pointers: row_ptr (n+1), col (m_dir
 * uint32 ids, symmetric CSR), labels_out (n uint32).  stream is a
 * cudaStream_t (NULL = default stream).  The call is synchronous: it waits on
 * `stream` until the solve is done and returns its status (CC_ERR_INVALID for
 * offsets that are not monotone or exceed m_dir, or an id >= n), so it cannot
 * be recorded into a CUDA graph by stream capture.  Scratch
 * lives in a fixed 4 MiB device array that every GPU loading the library
 * keeps until exit; graphs with min(n, m_dir/33 + 1) > 1,048,512 are rejected
 * with CC_ERR_UNSUPPORTED before any launch.  All calls share that array:
 * calls that overlap on the GPU race and must be serialised by the caller.
 * The first call on a device looks up the array's device address and is the
 * first launch of its kernels there, which CUDA's lazy module loading may
 * turn into an allocation and a synchronisation: make one warm-up call per
 * device before allocation becomes forbidden, and before any stream capture
 * begins on that device.
 */
int cc_gpu_run_noalloc(const uint64_t *row_ptr, const uint32_t *col, uint64_t n,
                       uint64_t m_dir, uint32_t *labels_out, void *stream);

/* ---- contexts ------------------------------------------------------------ */

/* Create a context on `device`.  stream may be NULL (the context creates a
   non-blocking stream) or a cudaStream_t owned by the caller. */
int cc_ctx_create(cc_ctx **out, int device, void *stream);
int cc_ctx_destroy(cc_ctx *ctx);
/* As cc_gpu_run on ctx's stream; labels_where says where labels_out lives. */
int cc_ctx_run(cc_ctx *ctx, const cc_csr *g, cc_algo algo,
               const cc_config *cfg, uint64_t seed, void *labels_out,
               uint32_t labels_where);
/*
 * Component-size summary of a label array (OutputComponents,
 * static_graph.h:504-591), on the device: the (size, number of components of
 * that size) pairs in ascending size, as 2 * min(*npairs, cap) words of
 * `pairs`, and in *num_components the number of components with more than one
 * vertex (the reference's "NUM COMPONENTS").  labels: n values below n (the
 * solvers' canonical labels), id_bytes 4 or 8, where CC_HOST or CC_DEVICE.
 * *npairs receives the number of distinct sizes (at most sqrt(2n) + 1; pairs
 * beyond cap are not written).  ctx NULL: the default context.
 */
int cc_component_sizes(cc_ctx *ctx, const void *labels, uint32_t id_bytes, uint32_t where, uint64_t n,
                       uint64_t *pairs, uint64_t cap, uint64_t *npairs, uint64_t *num_components);
/*
 * The seeded G(n, m) and 2D bond-percolation generators of cc_gen.h, run on
 * the device: the same graph as cc_gen_gnm / cc_gen_grid for the same
 * arguments (the same hash of (seed, index), the same sorted rows), written
 * into the caller's device buffers row_ptr (n + 1 offsets) and col (cap ids
 * of id_bytes); *m_dir receives the number of entries (CC_ERR_INVALID when it
 * exceeds cap; 4 X Y and 2 m always suffice).  ctx NULL: the default context.
 */
int cc_gen_grid_device(cc_ctx *ctx, uint64_t X, uint64_t Y, double p, uint64_t seed, uint32_t id_bytes,
                       uint64_t *row_ptr, void *col, uint64_t cap, uint64_t *m_dir);
int cc_gen_gnm_device(cc_ctx *ctx, uint64_t n, uint64_t m, uint64_t seed, uint32_t id_bytes,
                      uint64_t *row_ptr, void *col, uint64_t cap, uint64_t *m_dir);
/* The random hyperbolic graph of cc_gen_rhg (cc_gen.h), built on the device:
   the same CSR bit for bit (the model's per-point values and edge test are
   evaluated with the same correctly rounded operations on host and device).
   Stand-in for KaGen's rhg generator (lib/io/io_utils.h:72-73).  row_ptr:
   n+1 device words; col: cap device ids; *m_dir receives the number of
   directed entries (also when it exceeds cap, which gives CC_ERR_INVALID).
   Needs about 60 bytes of device scratch per vertex plus 16 per entry. */
int cc_gen_rhg_device(cc_ctx *ctx, uint64_t n, double avg_deg, double gamma, uint64_t seed,
                      uint32_t id_bytes, uint64_t *row_ptr, void *col, uint64_t cap,
                      uint64_t *m_dir);

/*
 * The reference's input files read straight into a device CSR: METIS text
 * (GraphIO::ReadMETISFile, lib/io/graph_io.h:281-382) and the sorted binary
 * edge file (GraphIO::ReadSortedBinaryFile, graph_io.h:910-1175).  The file's
 * bytes cross the host link once; tokens, keys, the sort and the rows are
 * built on the device, and the result is the CSR of cc_read_metis /
 * cc_read_binary_edges (cc_gen.h) bit for bit: symmetric, rows sorted,
 * self-loops and repeated edges dropped.  Size query: with row_ptr NULL only
 * the header is read and *n and *m_dir receive the vertex count and an upper
 * bound of the directed entries (nothing runs on the device).  Otherwise
 * row_ptr holds n+1 device words and col cap device ids; *m_dir receives the
 * entries (CC_ERR_INVALID when they exceed cap, or for an id outside [1, n]
 * or a malformed file).  METIS files below 4 GB.  ctx NULL: the default
 * context (its page-locked staging holds the file).
 */
int cc_read_metis_device(cc_ctx *ctx, const char *path, uint32_t id_bytes, uint64_t *row_ptr,
                         void *col, uint64_t cap, uint64_t *n, uint64_t *m_dir);
int cc_read_binary_edges_device(cc_ctx *ctx, const char *path, uint32_t id_bytes, uint64_t *row_ptr,
                                void *col, uint64_t cap, uint64_t *n, uint64_t *m_dir);

int cc_ctx_stats(cc_ctx *ctx, cc_stats *out);
/* Device bytes the context holds in its arena (grows on demand, reused). */
uint64_t cc_ctx_arena_bytes(cc_ctx *ctx);
/* Profiling, off by default.  `flags`: CC_PROF_KERNELS = per-kernel
   CUDA-event timing in cc_stats.kernels (adds event records between the
   kernels), CC_PROF_COMPONENTS = cc_stats.num_components (adds one counting
   pass over the labels and a readback per solve); 0 switches both off. */
enum { CC_PROF_KERNELS = 1, CC_PROF_COMPONENTS = 2 };
int cc_ctx_set_profiling(cc_ctx *ctx, int flags);
/* Per-kernel sums (launches, ms, bytes), solve_ms, total_ms, launch and byte
   counts over every solve since profiling was last switched on; *solves gets
   their number.  (new, no counterpart in the reference: lets a caller time
   many solves without reading statistics between them) */
int cc_ctx_profile_totals(cc_ctx *ctx, cc_stats *out, uint64_t *solves);
/* The cudaStream_t the context launches on. */
void *cc_ctx_stream(cc_ctx *ctx);

/* Schedule of the hook-and-compress pass (partition-local components, base
   cases, CC_ALLREDUCE).  Zero fields keep the defaults. */
enum { CC_HOOK_AUTO = 0, CC_HOOK_GLOBAL = 1, CC_HOOK_TILED = 2, CC_HOOK_SAMPLED = 3 };
typedef struct cc_tuning {
  uint32_t hook_mode;      /* CC_HOOK_*: GLOBAL links every edge (thread per
                              vertex); TILED unites each CTA tile in shared
                              memory first; SAMPLED links two neighbours per
                              vertex, then only rows outside the largest
                              component; AUTO picks TILED when a sample of rows
                              shows < 50 % tile-crossing edges and < 10 % of
                              edges in hub rows, GLOBAL when the graph fits in
                              96 MB (L2-resident) with < 10 % hub edges, else
                              SAMPLED */
  uint32_t tile_vertices;  /* vertices per CTA tile of the TILED pass, 2 bytes
                              of shared memory each (default 32768, 32 to
                              65536); SAMPLED's tiled link rounds use half as
                              many vertices, 4 bytes each */
  uint32_t tile_threads;   /* CTA size of the tiled pass (default 1024) */
  uint32_t hub_degree;     /* rows above are split into pieces of 2048 edges,
                              one warp per piece (default 32) */
} cc_tuning;
int cc_ctx_set_tuning(cc_ctx *ctx, const cc_tuning *t);
int cc_ctx_get_tuning(cc_ctx *ctx, cc_tuning *t);
/*
 * HOST graphs solved by sampled linking (CC_EXP with one rank, CC_ALLREDUCE,
 * when a sample of rows shows the link-round entries staying in their tiles):
 * with in_place = 1 (the default) and row_ptr and col in page-locked memory
 * (cudaHostAlloc / cudaHostRegister with the context's device current, mapped
 * into the device's address space),
 * the kernels read the offsets, each row's first entries and the rows outside
 * the giant component straight from the caller's buffers, and nothing else of
 * the ids crosses the host link; cc_stats.h2d_bytes then counts the offsets
 * and the first two entries a row (at most m_dir) that the link pass reads
 * (the link moves whole sectors around them).
 * in_place = 2: the ids are read in place and the offsets copied in chunks
 * (as one degree byte a row where they fit) under the link pass.
 * in_place = 0, or pageable buffers: the rows are copied to the device in
 * chunks under the link pass.  Labels are the same either way.  (new, no
 * counterpart in the reference: its input is in memory already)
 */
int cc_ctx_set_host_reads(cc_ctx *ctx, int in_place);

#ifdef __cplusplus
}
#endif

#endif /* CC_GPU_H_ */
