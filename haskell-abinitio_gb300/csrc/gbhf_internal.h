// Host-side context and internal interfaces of libgbhf.
#pragma once
#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gbhf.h"
#include "gbhf_common.cuh"

namespace gbhf {

// Per-context cache of device blocks.  cudaFree waits for the whole device,
// so a buffer released by one context (one stream) would stall every other
// context's work; instead released blocks go back to the pool of the context
// that allocated them and are handed out again to later allocations of the
// same context, whose work is ordered on the same stream.  Block sizes are
// rounded up to 256 bytes and then to four steps per power of two.  The
// blocks are freed when the context is destroyed (and all free blocks when an
// allocation fails).
struct DevPool {
  std::map<size_t, std::vector<void*>> free_blocks;
  std::vector<void*> all_blocks;
  std::mutex mu;
  static size_t round_size(size_t b) {
    b = (b + 255) & ~(size_t)255;
    size_t hi = 256;
    while (hi < b) hi <<= 1;
    if (hi <= 1024) return hi;
    const size_t step = hi >> 3;   // hi/2 < b <= hi: steps of hi/8
    return (b + step - 1) / step * step;
  }
  cudaError_t get(size_t bytes, void** out) {
    {
      std::lock_guard<std::mutex> lock(mu);
      auto it = free_blocks.find(bytes);
      if (it != free_blocks.end() && !it->second.empty()) {
        *out = it->second.back();
        it->second.pop_back();
        return cudaSuccess;
      }
    }
    cudaError_t e = cudaMalloc(out, bytes);
    if (e == cudaErrorMemoryAllocation) {
      (void)cudaGetLastError();
      trim();
      e = cudaMalloc(out, bytes);
    }
    if (e == cudaSuccess) {
      std::lock_guard<std::mutex> lock(mu);
      all_blocks.push_back(*out);
    }
    return e;
  }
  void put(void* p, size_t bytes) {
    std::lock_guard<std::mutex> lock(mu);
    free_blocks[bytes].push_back(p);
  }
  void trim() {
    std::lock_guard<std::mutex> lock(mu);
    for (auto& kv : free_blocks)
      for (void* p : kv.second) {
        cudaFree(p);
        for (auto& q : all_blocks)
          if (q == p) q = nullptr;
      }
    free_blocks.clear();
  }
  ~DevPool() {
    for (void* p : all_blocks)
      if (p) cudaFree(p);
  }
};

// An instantiated CUDA graph of a fixed launch sequence, rebuilt when the
// key (sizes and buffer addresses baked into the launches) changes.
struct GraphCache {
  cudaGraphExec_t exec = nullptr;
  std::vector<const void*> key;
  int launches = 0;   // kernels in one replay
  GraphCache() = default;
  GraphCache(const GraphCache&) = delete;
  GraphCache& operator=(const GraphCache&) = delete;
  ~GraphCache() { reset(); }
  void reset() {
    if (exec) cudaGraphExecDestroy(exec);
    exec = nullptr;
    key.clear();
  }
};

// Pool used by allocations on this thread: set by every entry point for the
// context it works on (PoolScope), null outside the library.
extern thread_local DevPool* tls_pool;

// Device buffer with RAII release (no copies); grows, never shrinks.
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  size_t bytes = 0;
  DevPool* owner = nullptr;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) {
      if (owner) owner->put(p, bytes);
      else cudaFree(p);
    }
    p = nullptr;
    n = 0;
    bytes = 0;
    owner = nullptr;
  }
  cudaError_t alloc(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    if (count == 0) count = 1;
    DevPool* pool = tls_pool;
    if (pool) {
      const size_t b = DevPool::round_size(count * sizeof(T));
      void* q = nullptr;
      cudaError_t e = pool->get(b, &q);
      if (e == cudaSuccess) {
        p = static_cast<T*>(q);
        n = b / sizeof(T);
        bytes = b;
        owner = pool;
      }
      return e;
    }
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
};

struct Shell {
  int atom, L, np, ncomp, f0;   // f0: first basis function (components contiguous: x,y,z; xx,xy,xz,yy,yz,zz)
  int mol = 0;                  // molecule of the shell (batched SCF); 0 for one molecule
  std::vector<double> expo, coef;   // coef: the first component's contraction coefficients
  double scale[6] = {1, 1, 1, 1, 1, 1};   // component c's coefficients = scale[c] * coef (d shells)
};

// Shell-pair classes (la >= lb): 0 (s,s), 1 (p,s), 2 (p,p), 3 (d,s), 4 (d,p), 5 (d,d).
constexpr int NPCLS = 6;
__host__ __device__ constexpr int pair_class_of(int la, int lb) { return la * (la + 1) / 2 + lb; }
// J/K quartet combos (one per unordered pair of pair classes): the six s/p classes first, then
// the fifteen with a d pair (warp-per-quartet kernels).
constexpr int NCOMBO = 21;
constexpr int NCOMBO_SP = 6;
// The s/p combos (pp|ss) and (pp|ps) run with the lower pair as the warp-shared
// bra ((ss|pp), (ps|pp)): their generated code defers the transformation of the
// per-lane, higher-momentum pair.
constexpr int COMBO_BRA[NCOMBO] = {0, 1, 1, 0, 1, 2, 3, 3, 3, 3, 4, 4, 4, 4, 4, 5, 5, 5, 5, 5, 5};
constexpr int COMBO_KET[NCOMBO] = {0, 0, 1, 2, 2, 2, 0, 1, 2, 3, 0, 1, 2, 3, 4, 0, 1, 2, 3, 4, 5};
// Gradient combos: every ordered (bra class, ket class); the nine s/p ones first.
constexpr int NCOMBO_MAX = 36;
constexpr int NGCOMBO_SP = 9;
constexpr int GRAD_COMBO_BRA[NCOMBO_MAX] = {0, 0, 0, 1, 1, 1, 2, 2, 2, 0, 0, 0, 1, 1, 1, 2, 2, 2,
                                            3, 3, 3, 3, 3, 3, 4, 4, 4, 4, 4, 4, 5, 5, 5, 5, 5, 5};
constexpr int GRAD_COMBO_KET[NCOMBO_MAX] = {0, 1, 2, 0, 1, 2, 0, 1, 2, 3, 4, 5, 3, 4, 5, 3, 4, 5,
                                            0, 1, 2, 3, 4, 5, 0, 1, 2, 3, 4, 5, 0, 1, 2, 3, 4, 5};

struct Segment {
  int start, end, K;   // global pair indices [start, end), primitive pairs per pair
  int data_off;        // offset of this segment's ket-layout primitive data
};

struct Basis {
  int natoms = 0, nbf = 0;
  std::vector<double> xyz, Z;
  // CGF description as given
  std::vector<int> cgf_atom, cgf_lxyz, cgf_nprim;
  std::vector<double> prim_coef, prim_exp;
  std::vector<int> cgf_off;
  std::vector<Shell> shells;
  int maxL = 0;
  bool shells_ok = false;   // every CGF grouped into a complete s or p shell
  std::string shell_msg;
  // molecules (batched SCF): atoms [mol_atom_off[m], mol_atom_off[m+1]) and
  // functions [mol_fn_off[m], mol_fn_off[m+1]) of molecule m; one molecule
  // otherwise.  No shell pair or quartet spans two molecules.
  int nmol = 1;
  std::vector<int> mol_atom_off, mol_fn_off;
  std::vector<long long> mol_moff;   // offset of molecule m's n_m x n_m block in a stacked matrix
  long long stacked = 0;             // sum of n_m^2
};

// Shell-pair data on the device, in the order used by the J/K kernels:
// class 0 pairs, then class 1, then class 2; inside a class grouped by
// primitive-pair count (segments), inside a segment by Schwarz bound descending.
struct PairData {
  int npairs = 0;
  int cls_start[NPCLS + 1] = {};
  std::vector<Segment> segs[NPCLS];
  std::vector<int> hA, hB, hK, hPoff, hSeg;  // host copies
  std::vector<double> hQ;
  DBuf<int> A, B, K, poff, kseg;             // kseg: segment index (global list)
  DBuf<double> Q;
  DBuf<float> Qf;                  // Q in FP32 (the FP32 kernels' per-quartet density test)
  DBuf<int4> seg_info;                       // (start, end, K, data_off) per segment, all classes
  int nseg_total = 0;
  int seg_cls_start[NPCLS + 1] = {};
  // molecules: pair -> molecule, and the ket segments of (class, molecule)
  // [mseg[2*(cls*nmol+m)], mseg[2*(cls*nmol+m)+1])
  DBuf<int> mol;
  DBuf<int> mseg;
  std::vector<int> hmseg;
  // primitive-pair data: bra layout (pair-contiguous) and ket layout
  // (segment-transposed: prim k of pair j at data_off + k*len + (j-start)).
  DBuf<double> bra64, ket64;   // BRA_NFIELD arrays of length nprimpairs each
  DBuf<float> bra32, ket32;
  size_t nprim_pairs = 0;
};

struct TaskLists {
  DBuf<int> item_count;    // per (combo, bra) item: [n64, n32]
  DBuf<int> item_off;      // exclusive scan
  DBuf<int> scan_part;     // per scan tile: sums, then their exclusive scan
  DBuf<int4> tasks64, tasks32;
  DBuf<int> ranges;        // per combo: start64, end64, start32, end32
  DBuf<int> counters;      // per combo & precision: work-queue heads
  DBuf<unsigned long long> stats;  // per combo: shell quartets, fn quartets, prim quartets (64, 32)
  bool stats_pending = false;      // stats holds counts of builds not yet added to the profile
  DBuf<int> ics_d, cls_d, scs_d;   // task generation inputs (live until its kernels have run)
  int nitems = 0;
  std::vector<int> combo_item_start;   // host: first item of each combo
  double thr_all = -1, thr64 = -1;     // thresholds the current lists were built for
  double thr_exact = 0;                // per-quartet density screening cutoff of the current build
  int ncombo = 0;
  int hranges[4 * NCOMBO_MAX] = {0};   // host copy of ranges
  DBuf<int> f0;                        // first basis function per shell
  DBuf<double> sscale;                 // per shell: 6 component scales (d shells; 1 otherwise)
  DBuf<int> nc;                        // components per shell
  DBuf<int> atom;                      // atom of each shell
  DBuf<int> smol;                      // molecule of each shell
  DBuf<int> mn;                        // per molecule: functions
  DBuf<long long> moff;                // per molecule: offset of its block in stacked matrices
  DBuf<int> fmol;                      // per function: molecule
  DBuf<int> amol;                      // per atom: molecule
  DBuf<int> mfo, mao;                  // per molecule: first function, first atom (nmol+1)
  DBuf<double> row, pw, pb, sw;        // density weights (incremental builds, gradient)
  long f0_gen = -1;                    // basis generation f0 was uploaded for
};

struct JacobiWork {
  DBuf<double> A, A2, V, rot, red, t1, t2, t3;
  DBuf<int> sweeps;
  DBuf<unsigned> bar;
  int grid = 0;
  int last_sweeps = 0;
};

// Work buffers of the tridiagonal eigen-solver (tridiag.cu).
struct TridiagWork {
  DBuf<double> d, e, e2, tau, lam, scal, Vt, Zt, Z2, S, M;
  DBuf<float> df, e2f;
  DBuf<int> blk, rank;
};
// Largest n of the tridiagonal path: the packed lower triangle of A plus two
// vectors in one CTA's shared memory (232: 215 KiB).  Larger n use Jacobi.
constexpr int TRIDIAG_MAX_N = 232;

struct Profile {
  bool events = false;
  double jk_ms64 = 0, jk_ms32 = 0, dense_ms = 0;
  double prim64 = 0, prim32 = 0, shellq = 0, fnq = 0;
  long long launches = 0;
  double cls[NCOMBO][2][4] = {};   // per combo and precision: shell q, fn q, prim q, ms
  // host wall-clock per SCF phase (ms): setup, Fock, DIIS, diagonalisation, other; Jacobi sweeps
  double ph_setup = 0, ph_fock = 0, ph_diis = 0, ph_diag = 0, ph_other = 0, jacobi_sweeps = 0, jacobi_calls = 0;
  double ph_grad = 0, batch_steps = 0, purify_steps = 0, purify_calls = 0, ph_pairs = 0;
  double gcls_ms[NCOMBO_MAX][2] = {};   // per gradient combo and precision: kernel ms (events mode)
};

}  // namespace gbhf

struct gbhf_ctx {
  gbhf::DevPool devpool;         // first member: destroyed after every buffer below
  int device = 0;
  int nsm = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  gbhf::Basis basis;
  bool have_grid = false;
  gbhf::DBuf<double> boys_ref;   // 15 x 1001 reference grid
  gbhf::DBuf<double> boys64;     // exact FP64 table
  gbhf::DBuf<float> boys32;      // exact FP32 table
  gbhf::DBuf<double> boysh64;    // Horner tables for the J/K kernels
  gbhf::DBuf<float> boysh32;
  // basis on device (function level, for 1-e integrals and canonical ERIs)
  gbhf::DBuf<double> d_xyz, d_Z, d_coef, d_exp;
  gbhf::DBuf<int> d_fn;          // per CGF: atom, lx, ly, lz, np, off (6 ints)
  bool basis_dev = false;
  long basis_gen = 0;            // incremented by every gbhf_set_basis
  gbhf::PairData pairs;
  bool pairs_ready = false;
  gbhf::TaskLists tasks;
  gbhf::TaskLists gtasks;        // gradient task lists
  const int* mol_active = nullptr;   // batched SCF: per molecule 0/1 (device); nullptr = all
  gbhf::GraphCache g_purify, g_bpurify;   // four purification steps (one molecule, batch)
  // shell pairs of the one-electron kernels, grouped by pair class (basis generation onee_gen)
  gbhf::DBuf<int2> onee_pairs;
  int onee_cls[gbhf::NPCLS + 1] = {};
  long onee_gen = -1;
  // dense work buffers (n*n doubles)
  gbhf::DBuf<double> w[24];
  gbhf::JacobiWork jac;
  gbhf::TridiagWork tri;
  size_t smem_optin = 0;          // largest dynamic shared memory per block (opt-in)
  bool force_jacobi = false;      // GBHF_EIGEN=jacobi at gbhf_create: every eigen-solve by Jacobi
  bool force_sytrd_single = false; // GBHF_EIGEN=single-cta: tridiagonalisation in one CTA
  int sytrd_cluster = 0;          // 1: the cluster tridiagonalisation runs here, -1: it does not, 0: not checked
  // state of the last SCF (for the gradient): density, Fock matrix, occupation
  gbhf::DBuf<double> last_D, last_F;
  // state of the last converged UHF SCF: alpha and beta densities, energy-weighted density
  gbhf::DBuf<double> last_uDa, last_uDb, last_uW;
  long last_ugen = -1;
  double grad_jcoef = 1.0;        // Coulomb weight in the gradient kernels' Gamma (0: exchange only)
  gbhf::DBuf<double> guess_D;        // gbhf_set_guess_density (flat), valid for basis generation guess_gen
  long guess_gen = -1;
  std::vector<double> scf_trace;     // per-step records of the last SCF (GBHF_SCF_TRACE_FIELDS each)
  int last_nocc = -1;
  long last_gen = -1;
  // worker contexts of gbhf_scf_batch (owned; destroyed with this context)
  std::vector<gbhf_ctx*> pool;
  // SAD guess: atomic densities by atom key, and the context that computes them
  std::map<std::string, std::vector<double>> sad_cache;
  gbhf_ctx* sad_ctx = nullptr;
  gbhf::DBuf<float> dfloat;
  gbhf::DBuf<int> dev_status;
  int purify_grid = 0;              // co-resident blocks of the fused purification kernel
  int tc2_grid = 0;                 // co-resident blocks of the one-barrier TC2 kernel
  bool purify_defer = false;        // purify leaves its check to the next reduce_stats (SCF loop)
  bool purify_pending = false;      // a purification record waits in small[PURIFY_REC..+2]
  int purify_ne = 0;                // electrons of the pending purification
  gbhf::DBuf<double> red_part;     // per-block partials of the grid reductions (k_stats_grid, k_dots, k_max_abs)
  gbhf::DBuf<unsigned> red_ticket; // their last-block ticket (zero between launches)
  gbhf::DBuf<unsigned> barrier;
  gbhf::DBuf<double> small;
  gbhf::Profile prof;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t evc[2 * gbhf::NCOMBO + 1] = {};   // per-class J/K launch boundaries (profiling)
  cudaEvent_t evu[8] = {};       // user slots (gbhf_event_record)
  cudaEvent_t evg[2 * gbhf::NCOMBO_MAX + 1] = {};   // per-combo gradient launch boundaries (profiling)
  cudaEvent_t evp[5] = {};       // SCF step phase boundaries (Fock, DIIS, density, convergence)
  // task budgets of the direct builds per quartet class (J/K) and class pair
  // (gradient): primitive quartets per lane and task, kets per task
  int jk_lp[gbhf::NCOMBO_MAX] = {}, jk_tk[gbhf::NCOMBO_MAX] = {};
  int gr_lp[gbhf::NCOMBO_MAX] = {}, gr_tk[gbhf::NCOMBO_MAX] = {};
  bool tuned[2] = {false, false};   // budgets chosen by the autotuner or the caller
  // side streams of the J/K build: the class kernels of one build run
  // concurrently so that the tail of one persistent launch overlaps the next
  // side streams for the J/K class launches (eight measured 1% faster than four on the
  // (H2O)16 mixed SCF); the gradient's class launches use the first NSIDE_GRAD (four: eight
  // were 3% slower there)
  static constexpr int NSIDE = 8;
  static constexpr int NSIDE_GRAD = 4;
  cudaStream_t side[NSIDE] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[NSIDE] = {};
  gbhf::DBuf<unsigned char> flush;
};

namespace gbhf {

// Makes `c`'s pool the allocation pool of this thread for the scope.
struct PoolScope {
  DevPool* prev;
  explicit PoolScope(gbhf_ctx* c) : prev(tls_pool) {
    if (c) tls_pool = &c->devpool;
  }
  ~PoolScope() { tls_pool = prev; }
};

// error helpers
gbhf_status fail(gbhf_ctx* c, gbhf_status s, const std::string& msg);
gbhf_status cuda_fail(gbhf_ctx* c, cudaError_t e, const char* where);
#define GBHF_CUDA(ctx, call)                                        \
  do {                                                              \
    cudaError_t e__ = (call);                                       \
    if (e__ != cudaSuccess) return gbhf::cuda_fail(ctx, e__, #call); \
  } while (0)
// The launch just issued (named by `what`) was accepted.
#define GBHF_LAUNCHED(ctx, what)                                      \
  do {                                                                \
    cudaError_t e__ = cudaGetLastError();                             \
    if (e__ != cudaSuccess) return gbhf::cuda_fail(ctx, e__, what);   \
  } while (0)
#define GBHF_TRY(call)                   \
  do {                                   \
    gbhf_status s__ = (call);            \
    if (s__ != GBHF_OK) return s__;      \
  } while (0)

inline void count_launch(gbhf_ctx* c, int n = 1) { c->prof.launches += n; }

// Capture `body` (launches on c->stream only, no synchronisation) into the cache
// unless the key matches the cached graph, then launch the graph once.
template <typename Body>
gbhf_status graph_run(gbhf_ctx* c, GraphCache& g, const std::vector<const void*>& key, Body body) {
  if (!g.exec || g.key != key) {
    g.reset();
    const long before = c->prof.launches;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamBeginCapture");
    const gbhf_status s = body();
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(c->stream, &graph);
    if (s != GBHF_OK) {
      if (graph) cudaGraphDestroy(graph);
      return s;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      g.exec = nullptr;
      return cuda_fail(c, e, "cudaGraphInstantiate");
    }
    g.key = key;
    g.launches = (int)(c->prof.launches - before);
    c->prof.launches = before;
  }
  const cudaError_t e = cudaGraphLaunch(g.exec, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphLaunch");
  count_launch(c, g.launches);
  return GBHF_OK;
}

// Work slot `slot` of the context with at least `count` doubles (nullptr on
// allocation failure).  Slots 0-9: SCF driver; 10-12: diagonalHF and
// symmOrtho; 13-14: DIIS error; 15-23: API entry points.
inline double* ws(gbhf_ctx* c, int slot, size_t count) {
  if (c->w[slot].alloc(count) != cudaSuccess) return nullptr;
  return c->w[slot].p;
}
#define GBHF_WS(ctx, var, slot, count)                                                      \
  double* var = gbhf::ws(ctx, slot, count);                                                 \
  if (!var) return gbhf::fail(ctx, GBHF_ERR_CUDA, "device allocation failed (work buffer)")

// setup.cu
// Several molecules at once: atom_off / cgf_off (nmol+1 entries) partition the
// atoms and CGFs; cgf_atom holds global atom indices.
gbhf_status build_basis_mols(gbhf_ctx* c, int n_atoms, const double* xyz, const double* Z, int n_cgf,
                             const int* cgf_atom, const int* cgf_lxyz, const int* cgf_nprim, const double* coef,
                             const double* expo, int nmol, const int* atom_off, const int* cgf_off);
gbhf_status build_basis(gbhf_ctx* c, int n_atoms, const double* xyz, const double* Z, int n_cgf,
                        const int* cgf_atom, const int* cgf_lxyz, const int* cgf_nprim, const double* coef,
                        const double* expo);
gbhf_status ensure_boys_tables(gbhf_ctx* c);
gbhf_status ensure_pairs(gbhf_ctx* c);

// onee.cu
gbhf_status onee_matrices(gbhf_ctx* c, bool ref, double* d_S, double* d_H);   // flat (N(N+1)/2), device
gbhf_status onee_stacked(gbhf_ctx* c, double* d_S, double* d_H);   // square blocks of every molecule (exact mode)
// eri_canon.cu
gbhf_status eri_canonical_dev(gbhf_ctx* c, bool ref, double* d_eri);
gbhf_status fock_canonical_dev(gbhf_ctx* c, const double* d_H, const double* d_D, const double* d_eri, double* d_F);
gbhf_status boys_dev(gbhf_ctx* c, bool ref, int mmax, int n, const double* d_x, double* d_out);
gbhf_status boys_ref_grid_dev(gbhf_ctx* c, double* d_grid);
// jk.cu
// G_acc (n*n) += sym(G''(D)), D square n*n.  w = screening weight.
// local_weights: screen and choose precision with per-pair |D| weights (D is a
// density change); otherwise a uniform weight `weight`.
gbhf_status ensure_shell_arrays(gbhf_ctx* c);
gbhf_status build_grad_tasks(gbhf_ctx* c, const double* d_D, double cutoff, double mixed_cutoff, int precision);
// with_j = false: exchange only, G = -K(D)/2 (the open-shell spin-density term).
// Add the J/K kernels' counters of the builds since the last call to the
// profile (one copy and one host synchronisation).
gbhf_status flush_jk_stats(gbhf_ctx* c);
gbhf_status jk_build(gbhf_ctx* c, const double* d_Dsq, double* d_G, int precision, double schwarz,
                     double mixed_cutoff, double weight, bool local_weights = false, bool with_j = true);
// Q of every pair in [cls_start[cl], cls_start[cl+1]) (pairs grouped by class,
// bra-layout primitive data at d_poff), FP64 class code.
gbhf_status schwarz_classes_dev(gbhf_ctx* c, const int* cls_start, const int* d_K, const int* d_poff,
                                const double* d_bra, long long npp, double* d_Q);
// jkd.cu / gradd.cu: the classes with a d pair (warp per shell quartet).
// Schwarz bounds of classes 3..5 (dA, dB: shells of each pair, same order).
gbhf_status schwarz_dclasses_dev(gbhf_ctx* c, const int* cls_start, const int* dA, const int* dB, const int* d_K,
                                 const int* d_poff, const double* d_bra, long long npp, double* d_Q);
// J/K launch of combo 6..20 (COMBO_BRA/COMBO_KET), precision 0 = FP64, 1 = FP32.
gbhf_status launch_jk_dclass(gbhf_ctx* c, cudaStream_t strm, int combo, int prec, const double* D64,
                             const float* D32, double* G, int ntask, int with_j);
// Gradient combos on the generated lane-per-ket kernels (grad.cu); the rest
// go to launch_grad_dclass.
bool grad_gen_combo(int k);
// Gradient launch of a combo 9..35 (GRAD_COMBO_BRA/GRAD_COMBO_KET) without generated code.
gbhf_status launch_grad_dclass(gbhf_ctx* c, cudaStream_t strm, int combo, int prec, const double* D64,
                               const float* D32, double* grad, int ntask);
// linalg.cu
// sym: C (square) is known to be symmetric; only its upper tiles are computed and mirrored.
gbhf_status gemm(gbhf_ctx* c, bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda,
                 const double* B, int ldb, double beta, double* C, int ldc, bool sym = false);
gbhf_status eigh(gbhf_ctx* c, int n, const double* d_A, double* d_evals, double* d_evecs, const double* d_V0);
// tridiag.cu: Householder + bisection + inverse iteration, n <= TRIDIAG_MAX_N
gbhf_status eigh_tridiag(gbhf_ctx* c, int n, const double* d_A, double* d_evals, double* d_evecs);
size_t tridiag_smem_bytes(int n);
gbhf_status flat_to_square(gbhf_ctx* c, int n, const double* d_flat, double* d_sq);
gbhf_status square_to_flat(gbhf_ctx* c, int n, const double* d_sq, double* d_flat);
gbhf_status symm_ortho_dev(gbhf_ctx* c, int n, const double* d_S, double* d_X);
// S^-1/2 by Newton-Schulz (GEMMs only); density by canonical purification.
gbhf_status inv_sqrt_dev(gbhf_ctx* c, int n, const double* d_S, double* d_X, int* iters);
gbhf_status purify(gbhf_ctx* c, int n, int ne, const double* d_F, double* d_P, double* err_out, bool tc2 = true);
gbhf_status density_purified_dev(gbhf_ctx* c, int n, const double* d_Fsq, const double* d_X, int nocc,
                                 double* d_Dsq);
gbhf_status diagonal_hf_dev(gbhf_ctx* c, int n, const double* d_Fsq, const double* d_X, int nocc, double* d_C,
                            double* d_Dsq, double* d_eps, double* d_Cprime_warm);
gbhf_status diis_error_dev(gbhf_ctx* c, int n, const double* d_F, const double* d_S, const double* d_D,
                           const double* d_X, double* d_e);
gbhf_status gauss_elem_dev_call(gbhf_ctx* c, int m, const double* h_a, const double* h_b, double* h_x, bool* ok);
// scf.cu
gbhf_status scf_run(gbhf_ctx* c, const gbhf_scf_opts* o, gbhf_result* r);
gbhf_status uhf_run(gbhf_ctx* c, const gbhf_scf_opts* o, int multiplicity, gbhf_uhf_result* r);   // uhf.cu
// bscf.cu: the SCFs of every molecule of the context's basis (batched);
// energies / iterations / converged per molecule, grads 3 x total atoms (or nullptr)
gbhf_status bscf_run(gbhf_ctx* c, const gbhf_scf_opts* o, double* energies, int* iterations, int* converged,
                     double* grads);
// sad.cu: superposition-of-atomic-densities guess (n x n square, device)
gbhf_status sad_density(gbhf_ctx* c, double* d_D);
// Task budgets (tune.cu, jk.cu): defaults, the lane-per-ket test, the
// autotuner, and the two-electron gradient alone (for the autotuner).
void default_budgets(gbhf_ctx* c, int which);
bool lane_per_ket(int which, int k);
gbhf_status autotune_dev(gbhf_ctx* c, int which, const double* d_D, int precision, double schwarz,
                         double mixed_cutoff, int reps, double* class_ms);
gbhf_status gradient_uhf_dev(gbhf_ctx* c, const double* d_Da, const double* d_Db, const double* d_W, double schwarz,
                             double mixed_cutoff, int precision, double* d_grad);
gbhf_status grad_2e(gbhf_ctx* c, const double* d_D, double schwarz, double mixed_cutoff, int precision,
                    double* d_grad);
// grad.cu: D, W square on the device; gradient (3*natoms) on the device
gbhf_status gradient_dev(gbhf_ctx* c, const double* d_D, const double* d_W, double schwarz, double mixed_cutoff,
                         int precision, double* d_grad);
gbhf_status energy_weighted_density(gbhf_ctx* c, int n, int nocc, const double* d_C, const double* d_eps,
                                    double* d_W);
gbhf_status dot_matrices(gbhf_ctx* c, int n2, int k, const double* const* mats, const double* d_e,
                         double* d_out);
gbhf_status lincomb(gbhf_ctx* c, int n2, int k, const double* const* mats, const double* coefs, double* d_out);
gbhf_status reduce_stats(gbhf_ctx* c, int n, const double* d_e, const double* d_H, const double* d_F,
                         const double* d_Dnew, const double* d_Dold, double* host_out4);
gbhf_status axpby(gbhf_ctx* c, size_t n, double a, const double* x, double b, const double* y, double* out);
gbhf_status add_sym(gbhf_ctx* c, int n, const double* d_H, const double* d_Gpp, double* d_out);
gbhf_status max_abs(gbhf_ctx* c, size_t n, const double* d_x, double* host_out);
// Purification record slots in c->small and its checks (the deferred one runs
// in reduce_stats; purify_flush reads a pending one on its own).  c->small holds
// the statistics in 0-3, max|x| in 8, this record in 12-14, the Gauss
// elimination's operands from 16 on.
constexpr int PURIFY_REC = 12;
gbhf_status purify_finish(gbhf_ctx* c, const double* rec);
gbhf_status purify_flush(gbhf_ctx* c);
gbhf_status max_abs_dev(gbhf_ctx* c, size_t n, const double* d_x, double* d_out);   // into device memory
gbhf_status to_float(gbhf_ctx* c, size_t n, const double* d_x, float* d_y);

}  // namespace gbhf
