// Batched time stepping: many independent grids of uneven sizes advanced by one
// persistent kernel launch per fused pass, the whole time loop replayed from a
// captured CUDA graph.
//
// The reference advances one grid per process and schedules its temporal
// blocks with a dynamic ready queue over thread groups (diamond_ts.c:663-747).
// Here the unit of scheduling is a work item = (grid, x-y tile, z chunk) of one
// fused pass; CTAs pull items from an atomic counter, largest items first, so
// grids of very different sizes share the GPU without per-grid launch gaps or
// tail effects.  No CTA ever waits on another CTA.
//
// Each grid is an ordinary girih_gpu_ctx (upload, seeding, download and
// comparison go through the single-grid calls); the batch only owns the plan
// (per-launch grid arguments, item lists, counters) and the graph.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "context.cuh"
#include "fused_impl.cuh"

namespace girih {
namespace {

constexpr int kBatchThreads = 512;

template <class T> struct BatchGridArgs {
  FusedArgs<T> a;
  int op, tt;
};

// Thread mappings of the persistent kernel (512 threads): radius 1 = x pairs,
// 32x16 threads, 2 rows each (64 x 32 region); radius 4 = 64x8 threads, 4 rows
// each (64 x 32 region).  Both give the tiles of fused variant 0.
template <int OP> struct BatchMap;
template <> struct BatchMap<1> { static constexpr int NTX = 32, NTY = 16, CY = 2, VX = 2, TMAX = 4; };
template <> struct BatchMap<8> { static constexpr int NTX = 32, NTY = 16, CY = 2, VX = 2, TMAX = 4; };
template <> struct BatchMap<0> { static constexpr int NTX = 64, NTY = 8, CY = 4, VX = 1, TMAX = 2; };

template <class T> constexpr int batch_tmax(int r) { return r == 4 ? 2 : (sizeof(T) == 8 ? 2 : 4); }

template <int OP, class T, bool COMP, int TT>
__device__ __forceinline__ void run_tile(const FusedArgs<T> &a, int4 w, int tid, unsigned char *sm) {
  using M = BatchMap<OP>;
  if constexpr (OpTraits<OP>::R == 4 && TT == 1 && sizeof(T) == 4) {
    // radius 4, depth 1: x quads, 16x32 threads, one row each -- the same 64 x 32
    // region and output tile (the quads' 4-column alignment costs no column)
    fused_tile<OP, T, COMP, TT, 16, 32, 1, 4>(a, w.y, w.z, w.w, tid % 16, tid / 16, sm);
  } else {
    fused_tile<OP, T, COMP, TT, M::NTX, M::NTY, M::CY, M::VX>(a, w.y, w.z, w.w, tid % M::NTX, tid / M::NTX, sm);
  }
}

template <class T, bool COMP>
__global__ void __launch_bounds__(kBatchThreads) batched_pass(const BatchGridArgs<T> *__restrict__ args,
                                                              const int4 *__restrict__ items, int n_items,
                                                              unsigned *counter) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ BatchGridArgs<T> sa;
  __shared__ int s_item;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) s_item = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int it = s_item;
    if (it >= n_items) return;  // uniform over the CTA
    const int4 w = items[it];
    {  // the grid's arguments, once per item, into shared memory
      const unsigned *src = reinterpret_cast<const unsigned *>(args + w.x);
      unsigned *dst = reinterpret_cast<unsigned *>(&sa);
      for (int k = tid; k < (int)(sizeof(BatchGridArgs<T>) / 4); k += kBatchThreads) dst[k] = src[k];
    }
    __syncthreads();
    const int key = sa.op * 16 + sa.tt;
    if constexpr (sizeof(T) == 4) {
      switch (key) {
        case 8 * 16 + 1: run_tile<8, T, COMP, 1>(sa.a, w, tid, smraw); break;
        case 8 * 16 + 2: run_tile<8, T, COMP, 2>(sa.a, w, tid, smraw); break;
        case 8 * 16 + 3: run_tile<8, T, COMP, 3>(sa.a, w, tid, smraw); break;
        case 8 * 16 + 4: run_tile<8, T, COMP, 4>(sa.a, w, tid, smraw); break;
        case 1 * 16 + 1: run_tile<1, T, COMP, 1>(sa.a, w, tid, smraw); break;
        case 1 * 16 + 2: run_tile<1, T, COMP, 2>(sa.a, w, tid, smraw); break;
        case 1 * 16 + 3: run_tile<1, T, COMP, 3>(sa.a, w, tid, smraw); break;
        case 1 * 16 + 4: run_tile<1, T, COMP, 4>(sa.a, w, tid, smraw); break;
        case 0 * 16 + 1: run_tile<0, T, COMP, 1>(sa.a, w, tid, smraw); break;
        case 0 * 16 + 2: run_tile<0, T, COMP, 2>(sa.a, w, tid, smraw); break;
      }
    } else {
      switch (key) {
        case 8 * 16 + 1: run_tile<8, T, COMP, 1>(sa.a, w, tid, smraw); break;
        case 8 * 16 + 2: run_tile<8, T, COMP, 2>(sa.a, w, tid, smraw); break;
        case 1 * 16 + 1: run_tile<1, T, COMP, 1>(sa.a, w, tid, smraw); break;
        case 1 * 16 + 2: run_tile<1, T, COMP, 2>(sa.a, w, tid, smraw); break;
        case 0 * 16 + 1: run_tile<0, T, COMP, 1>(sa.a, w, tid, smraw); break;
        case 0 * 16 + 2: run_tile<0, T, COMP, 2>(sa.a, w, tid, smraw); break;
      }
    }
    __syncthreads();  // before s_item and sa are reused
  }
}

template <class T, bool COMP> size_t batched_smem() {
  size_t m = 0;
  auto upd = [&](size_t b) { m = b > m ? b : m; };
  if constexpr (sizeof(T) == 4) {
    upd(FusedShape<8, T, COMP, 4, 32, 16, 2, 2>::smem_bytes);
    upd(FusedShape<1, T, COMP, 4, 32, 16, 2, 2>::smem_bytes);
  } else {
    upd(FusedShape<8, T, COMP, 2, 32, 16, 2, 2>::smem_bytes);
    upd(FusedShape<1, T, COMP, 2, 32, 16, 2, 2>::smem_bytes);
  }
  upd(FusedShape<0, T, COMP, 2, 64, 8, 4, 1>::smem_bytes);
  upd(FusedShape<0, T, COMP, 1, 16, 32, 1, 4>::smem_bytes);
  return m;
}

template <class T, bool COMP>
cudaError_t launch_batched(const void *args, const int4 *items, int n_items, unsigned *counter, int nctas,
                           cudaStream_t st) {
  auto kern = batched_pass<T, COMP>;
  const size_t smem = batched_smem<T, COMP>();
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<nctas, kBatchThreads, smem, st>>>(static_cast<const BatchGridArgs<T> *>(args), items, n_items, counter);
  return cudaGetLastError();
}

template <class T, bool COMP> int batched_occupancy() {
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batched_pass<T, COMP>, kBatchThreads, batched_smem<T, COMP>());
  return occ < 1 ? 1 : occ;
}

int fail_b(int code, const std::string &msg) {
  set_error(msg);
  return code;
}

#define B_CK(...)                                                             \
  do {                                                                        \
    cudaError_t e_ = (__VA_ARGS__);                                           \
    if (e_ != cudaSuccess) {                                                  \
      set_error(std::string(#__VA_ARGS__) + ": " + cudaGetErrorString(e_));   \
      return GIRIH_GPU_ECUDA;                                                 \
    }                                                                         \
  } while (0)

}  // namespace
}  // namespace girih

using namespace girih;

struct girih_gpu_batch {
  int n = 0, device = 0, precision = 0, tsz = 4;
  std::vector<girih_gpu_ctx *> grids;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  // persistent plan and graph
  void *d_args = nullptr;
  int4 *d_items = nullptr;
  unsigned *d_counters = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int g_steps = -1;
  std::vector<int> g_start, g_end;  // per grid (iu1, iu2) before and after the cached loop
  int g_launches = 0, g_items = 0;
  // looped baseline graph
  cudaGraphExec_t lexec = nullptr;
  int l_steps = -1;
  std::vector<int> l_start, l_end;
  int l_launches = 0;
  int last_launches = 0, last_items = 0;
};

namespace {

void drop_plan(girih_gpu_batch *b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->g_steps = -1;
  if (b->d_args) cudaFree(b->d_args);
  if (b->d_items) cudaFree(b->d_items);
  if (b->d_counters) cudaFree(b->d_counters);
  b->d_args = nullptr;
  b->d_items = nullptr;
  b->d_counters = nullptr;
  if (b->lexec) cudaGraphExecDestroy(b->lexec);
  b->lexec = nullptr;
  b->l_steps = -1;
}

std::vector<int> rotation(girih_gpu_batch *b) {
  std::vector<int> r;
  for (auto *c : b->grids) {
    r.push_back(c->iu1);
    r.push_back(c->iu2);
  }
  return r;
}

void set_rotation(girih_gpu_batch *b, const std::vector<int> &r) {
  for (int g = 0; g < b->n; g++) {
    b->grids[g]->iu1 = r[2 * g];
    b->grids[g]->iu2 = r[2 * g + 1];
  }
}

// Fused depth a grid runs with in the persistent kernel.
int batch_depth(const girih_gpu_ctx *c) {
  const int tmax = c->tsz == 8 ? 2 : (c->g.r == 4 ? 2 : 4);
  int t = c->fcfg.depth > 0 ? c->fcfg.depth : 1;
  return t > tmax ? tmax : t;
}

template <class T>
void fill_args(BatchGridArgs<T> &ga, const girih_gpu_ctx *c, int prev, int cur, int oprev, int ocur, int tt,
               int write_prev, int zchunk) {
  std::memset(&ga, 0, sizeof(ga));
  ga.a.g = c->g;
  ga.a.prev = static_cast<const T *>(c->f[prev]);
  ga.a.cur = static_cast<const T *>(c->f[cur]);
  ga.a.roc2 = static_cast<const T *>(c->roc2);
  ga.a.out_prev = static_cast<T *>(c->f[oprev]);
  ga.a.out_cur = static_cast<T *>(c->f[ocur]);
  for (int m = 0; m < 5; m++) ga.a.cc[m] = c->cc[m];
  split_coefs(ga.a.cc, ga.a.cch, ga.a.ccl);
  ga.a.zchunk = zchunk;
  ga.a.write_prev = write_prev;
  ga.a.range_flag = reinterpret_cast<unsigned *>(c->acc + 6);  // the grid's error word
  ga.op = c->g.op;
  ga.tt = tt;
}

// Build the per-launch plan of `steps` steps from the current rotation and
// capture memset + persistent launches into a graph.
template <class T, bool COMP> int build_plan(girih_gpu_batch *b, int steps) {
  const int n = b->n;
  std::vector<BatchGridArgs<T>> args;
  std::vector<int4> items;
  std::vector<int> off, cnt;
  std::vector<int> rem(n, steps), iu1(n), iu2(n);
  for (int g = 0; g < n; g++) {
    iu1[g] = b->grids[g]->iu1;
    iu2[g] = b->grids[g]->iu2;
  }
  int launches = 0;
  for (;;) {
    bool any = false;
    for (int g = 0; g < n; g++) any |= rem[g] > 0;
    if (!any) break;
    const size_t base = args.size();
    args.resize(base + n);
    struct Item {
      int4 w;
      double cost;
    };
    std::vector<Item> li;
    for (int g = 0; g < n; g++) {
      girih_gpu_ctx *c = b->grids[g];
      BatchGridArgs<T> &ga = args[base + g];
      std::memset(&ga, 0, sizeof(ga));
      if (rem[g] <= 0) continue;
      const int tt = std::min(batch_depth(c), rem[g]);
      int spare[2], k = 0;
      for (int q = 0; q < 4 && k < 2; q++)
        if (q != iu1[g] && q != iu2[g]) spare[k++] = q;
      const int write_prev = (c->g.to == 2 || rem[g] == tt) ? 1 : 0;
      const Geom &gg = c->g;
      const int zchunk = std::min(gg.nz, 64);
      fill_args(ga, c, iu1[g], iu2[g], spare[0], spare[1], tt, write_prev, zchunk);
      FusedConfig fc = make_fused_config(gg, c->d.precision, tt, 0);  // tile of variant 0
      const int gx = (gg.nx + fc.bx - 1) / fc.bx, gy = (gg.ny + fc.by - 1) / fc.by;
      const int gz = (gg.nz + zchunk - 1) / zchunk;
      for (int z = 0; z < gz; z++) {
        const int zlen = std::min(zchunk, gg.nz - z * zchunk);
        const double cost = (double)(zlen + tt * (2 * gg.r + 1)) * tt * (gg.r == 4 ? 4.0 : 1.0);
        for (int y = 0; y < gy; y++)
          for (int x = 0; x < gx; x++) li.push_back({make_int4(g, x, y, z), cost});
      }
      iu1[g] = spare[0];
      iu2[g] = spare[1];
      rem[g] -= tt;
    }
    std::stable_sort(li.begin(), li.end(), [](const Item &p, const Item &q) { return p.cost > q.cost; });
    off.push_back((int)items.size());
    cnt.push_back((int)li.size());
    for (auto &it : li) items.push_back(it.w);
    launches++;
  }
  drop_plan(b);
  if (launches == 0) {
    b->g_steps = steps;
    b->g_start = rotation(b);
    b->g_end = b->g_start;
    b->g_launches = 0;
    b->g_items = 0;
    return 0;
  }
  B_CK(cudaMalloc(&b->d_args, args.size() * sizeof(BatchGridArgs<T>)));
  B_CK(cudaMalloc(&b->d_items, std::max<size_t>(1, items.size()) * sizeof(int4)));
  B_CK(cudaMalloc(&b->d_counters, launches * sizeof(unsigned)));
  B_CK(cudaMemcpyAsync(b->d_args, args.data(), args.size() * sizeof(BatchGridArgs<T>), cudaMemcpyHostToDevice, b->st));
  if (!items.empty())
    B_CK(cudaMemcpyAsync(b->d_items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice, b->st));
  B_CK(cudaStreamSynchronize(b->st));
  int nsm = 152;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->device);
  const int nctas = nsm * batched_occupancy<T, COMP>();
  cudaGraph_t graph = nullptr;
  B_CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeRelaxed));
  cudaError_t ce = cudaMemsetAsync(b->d_counters, 0, launches * sizeof(unsigned), b->st);
  for (int k = 0; k < launches && ce == cudaSuccess; k++)
    ce = launch_batched<T, COMP>(static_cast<BatchGridArgs<T> *>(b->d_args) + (size_t)k * n, b->d_items + off[k],
                                 cnt[k], b->d_counters + k, std::min(nctas, std::max(1, cnt[k])), b->st);
  cudaError_t ee = cudaStreamEndCapture(b->st, &graph);
  if (ce != cudaSuccess || ee != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return fail_b(GIRIH_GPU_ECUDA, std::string("batched graph capture: ") +
                                       cudaGetErrorString(ce != cudaSuccess ? ce : ee));
  }
  ce = cudaGraphInstantiate(&b->gexec, graph, 0);
  cudaGraphDestroy(graph);
  if (ce != cudaSuccess) {
    b->gexec = nullptr;
    return fail_b(GIRIH_GPU_ECUDA, std::string("batched graph instantiate: ") + cudaGetErrorString(ce));
  }
  b->g_steps = steps;
  b->g_start = rotation(b);
  b->g_end.clear();
  for (int g = 0; g < n; g++) {
    b->g_end.push_back(iu1[g]);
    b->g_end.push_back(iu2[g]);
  }
  b->g_launches = launches;
  b->g_items = (int)items.size();
  return 0;
}

int timed_graph(girih_gpu_batch *b, cudaGraphExec_t ex, float *ms_out) {
  if (GIRIH_CHECKED)  // every grid's error word starts clear
    for (auto *c : b->grids) B_CK(cudaMemsetAsync(c->acc + 6, 0, sizeof(unsigned), b->st));
  B_CK(cudaEventRecord(b->e0, b->st));
  if (ex) B_CK(cudaGraphLaunch(ex, b->st));
  B_CK(cudaEventRecord(b->e1, b->st));
  B_CK(cudaEventSynchronize(b->e1));
  B_CK(cudaGetLastError());
  float ms = 0;
  B_CK(cudaEventElapsedTime(&ms, b->e0, b->e1));
  if (ms_out) *ms_out = ms;
  if (GIRIH_CHECKED) {
    for (auto *c : b->grids) {
      unsigned bad = 0;
      B_CK(cudaMemcpy(&bad, c->acc + 6, sizeof(bad), cudaMemcpyDeviceToHost));
      if (bad & kFlagBounds) return fail_b(GIRIH_GPU_EBOUNDS, "a kernel index left its array or shared block");
    }
  }
  return 0;
}

struct BatchDevice {
  int prev = -1;
  explicit BatchDevice(int dev) {
    cudaGetDevice(&prev);
    if (prev != dev) cudaSetDevice(dev);
  }
  ~BatchDevice() {
    int cur = -1;
    cudaGetDevice(&cur);
    if (prev >= 0 && cur != prev) cudaSetDevice(prev);
  }
};

}  // namespace

extern "C" {

int girih_gpu_batch_create(girih_gpu_batch **out, int n, const girih_gpu_desc *descs) {
  if (!out || !descs || n < 1) return fail_b(GIRIH_GPU_EINVAL, "null argument or empty batch");
  *out = nullptr;
  for (int g = 0; g < n; g++) {
    const girih_gpu_desc &d = descs[g];
    if (d.target_kernel != 0 && d.target_kernel != 1 && d.target_kernel != 8)
      return fail_b(GIRIH_GPU_EUNSUPPORTED, "batched grids use the fused operators 0, 1 and 8");
    if (d.precision != descs[0].precision || d.device != descs[0].device)
      return fail_b(GIRIH_GPU_EINVAL, "all grids of a batch share one precision and one device");
    if (d.exact) return fail_b(GIRIH_GPU_EUNSUPPORTED, "exact rounding is provided by the plain schedule only");
  }
  girih_gpu_batch *b = new (std::nothrow) girih_gpu_batch;
  if (!b) return fail_b(GIRIH_GPU_ENOMEM, "host allocation failed");
  b->n = n;
  b->device = descs[0].device;
  b->precision = descs[0].precision;
  b->tsz = b->precision == GIRIH_FP64 ? 8 : 4;
  for (int g = 0; g < n; g++) {
    girih_gpu_desc d = descs[g];
    d.schedule = GIRIH_SCHED_FUSED;
    girih_gpu_ctx *c = nullptr;
    int e = girih_gpu_create(&c, &d);
    if (e) {
      girih_gpu_batch_destroy(b);
      return e;
    }
    b->grids.push_back(c);
  }
  BatchDevice bd(b->device);
  if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&b->e0) != cudaSuccess || cudaEventCreate(&b->e1) != cudaSuccess) {
    cudaGetLastError();
    girih_gpu_batch_destroy(b);
    return fail_b(GIRIH_GPU_ECUDA, "stream/event creation failed");
  }
  *out = b;
  return 0;
}

void girih_gpu_batch_destroy(girih_gpu_batch *b) {
  if (!b) return;
  {
    BatchDevice bd(b->device);
    if (b->st) cudaStreamSynchronize(b->st);
    drop_plan(b);
    if (b->e0) cudaEventDestroy(b->e0);
    if (b->e1) cudaEventDestroy(b->e1);
    if (b->st) cudaStreamDestroy(b->st);
  }
  for (auto *c : b->grids) girih_gpu_destroy(c);
  delete b;
}

girih_gpu_ctx *girih_gpu_batch_grid(girih_gpu_batch *b, int g) {
  if (!b || g < 0 || g >= b->n) return nullptr;
  return b->grids[g];
}

int girih_gpu_batch_autotune(girih_gpu_batch *b, int trial_steps) {
  if (!b) return fail_b(GIRIH_GPU_EINVAL, "null batch");
  BatchDevice bd(b->device);
  // one representative grid per (operator, size class) times every depth with
  // the tile of the persistent kernel; the fastest depth goes to the whole class
  std::vector<int> done(b->n, 0);
  for (int g = 0; g < b->n; g++) {
    if (done[g]) continue;
    girih_gpu_ctx *c = b->grids[g];
    if (!c->uploaded) return fail_b(GIRIH_GPU_ESTATE, "autotune before upload");
    const Geom &gg = c->g;
    auto cls_of = [](const Geom &q) {
      const double pts = (double)q.nx * q.ny * q.nz;
      return (int)std::floor(std::log2(pts > 1 ? pts : 1));
    };
    const int cls = cls_of(gg);
    // back up the state: tuning runs advance the grid
    const size_t fb = (size_t)gg.elems * c->tsz;
    void *bk[2] = {nullptr, nullptr};
    if (cudaMalloc(&bk[0], fb) != cudaSuccess || cudaMalloc(&bk[1], fb) != cudaSuccess) {
      cudaGetLastError();
      if (bk[0]) cudaFree(bk[0]);
      return fail_b(GIRIH_GPU_ENOMEM, "autotune backup allocation failed");
    }
    B_CK(cudaMemcpyAsync(bk[0], c->f[c->iu1], fb, cudaMemcpyDeviceToDevice, c->st));
    B_CK(cudaMemcpyAsync(bk[1], c->f[c->iu2], fb, cudaMemcpyDeviceToDevice, c->st));
    float best = 1e30f;
    int best_t = 1;
    const int tmax = c->tsz == 8 ? 2 : (gg.r == 4 ? 2 : 4);
    const int steps = trial_steps > 0 ? trial_steps : 12;
    for (int t = 1; t <= tmax; t++) {
      FusedConfig fc = make_fused_config(gg, c->d.precision, t, 0);
      if (!fc.depth) continue;
      c->fcfg = fc;
      if (c->gexec) cudaGraphExecDestroy(c->gexec);  // the context's cached loop used the old depth
      c->gexec = nullptr;
      c->g_steps = -1;
      float ms_min = 1e30f;
      for (int rep = 0; rep < 3; rep++) {
        float ms = 0;
        int e = girih_gpu_run(c, steps, &ms);
        if (e) {
          cudaFree(bk[0]);
          cudaFree(bk[1]);
          return e;
        }
        if (rep) ms_min = std::min(ms_min, ms);
      }
      if (ms_min < best) {
        best = ms_min;
        best_t = t;
      }
    }
    B_CK(cudaMemcpyAsync(c->f[0], bk[0], fb, cudaMemcpyDeviceToDevice, c->st));
    B_CK(cudaMemcpyAsync(c->f[1], bk[1], fb, cudaMemcpyDeviceToDevice, c->st));
    B_CK(cudaStreamSynchronize(c->st));
    cudaFree(bk[0]);
    cudaFree(bk[1]);
    c->iu1 = 0;
    c->iu2 = 1;
    for (int h = g; h < b->n; h++) {
      girih_gpu_ctx *o = b->grids[h];
      if (o->g.op == gg.op && cls_of(o->g) == cls) {
        o->fcfg = make_fused_config(o->g, o->d.precision, best_t, 0);
        if (o->gexec) cudaGraphExecDestroy(o->gexec);
        o->gexec = nullptr;
        o->g_steps = -1;
        done[h] = 1;
      }
    }
  }
  drop_plan(b);
  return 0;
}

int girih_gpu_batch_run(girih_gpu_batch *b, int nt, float *ms_out) {
  if (!b) return fail_b(GIRIH_GPU_EINVAL, "null batch");
  if (nt < 0) return fail_b(GIRIH_GPU_EINVAL, "nt must be >= 0");
  for (auto *c : b->grids)
    if (!c->uploaded) return fail_b(GIRIH_GPU_ESTATE, "run before upload");
  BatchDevice bd(b->device);
  for (auto *c : b->grids) cudaStreamSynchronize(c->st);
  const int steps = 2 * ((nt + 1) / 2);
  if (!b->gexec || b->g_steps != steps || b->g_start != rotation(b)) {
    int e = b->precision == GIRIH_FP64   ? build_plan<double, false>(b, steps)
            : b->precision == GIRIH_MIXED ? build_plan<float, true>(b, steps)
                                          : build_plan<float, false>(b, steps);
    if (e) return e;
  }
  int e = timed_graph(b, b->gexec, ms_out);
  if (e) return e;
  set_rotation(b, b->g_end);
  for (auto *c : b->grids) c->last_steps = steps;
  b->last_launches = b->g_launches;
  b->last_items = b->g_items;
  return 0;
}

int girih_gpu_batch_run_looped(girih_gpu_batch *b, int nt, float *ms_out) {
  if (!b) return fail_b(GIRIH_GPU_EINVAL, "null batch");
  if (nt < 0) return fail_b(GIRIH_GPU_EINVAL, "nt must be >= 0");
  for (auto *c : b->grids)
    if (!c->uploaded) return fail_b(GIRIH_GPU_ESTATE, "run before upload");
  BatchDevice bd(b->device);
  for (auto *c : b->grids) cudaStreamSynchronize(c->st);
  const int steps = 2 * ((nt + 1) / 2);
  if (!b->lexec || b->l_steps != steps || b->l_start != rotation(b)) {
    if (b->lexec) cudaGraphExecDestroy(b->lexec);
    b->lexec = nullptr;
    std::vector<int> start = rotation(b), end;
    int total = 0;
    cudaGraph_t graph = nullptr;
    B_CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeRelaxed));
    int err = 0;
    for (int g = 0; g < b->n && !err; g++) {
      girih_gpu_ctx *c = b->grids[g];
      int l = 0, a = c->iu1, bb = c->iu2;
      err = issue_steps_on(c, steps, &l, &a, &bb, b->st);
      end.push_back(a);
      end.push_back(bb);
      total += l;
    }
    cudaError_t ee = cudaStreamEndCapture(b->st, &graph);
    if (err || ee != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return err ? err : fail_b(GIRIH_GPU_ECUDA, std::string("looped capture: ") + cudaGetErrorString(ee));
    }
    cudaError_t ce = cudaGraphInstantiate(&b->lexec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) {
      b->lexec = nullptr;
      return fail_b(GIRIH_GPU_ECUDA, std::string("looped graph instantiate: ") + cudaGetErrorString(ce));
    }
    b->l_steps = steps;
    b->l_start = start;
    b->l_end = end;
    b->l_launches = total;
  }
  int e = timed_graph(b, b->lexec, ms_out);
  if (e) return e;
  set_rotation(b, b->l_end);
  b->last_launches = b->l_launches;
  b->last_items = 0;
  return 0;
}

int girih_gpu_batch_info(girih_gpu_batch *b, int *launches_last_run, int *items_last_run, int *depths) {
  if (!b) return fail_b(GIRIH_GPU_EINVAL, "null batch");
  if (launches_last_run) *launches_last_run = b->last_launches;
  if (items_last_run) *items_last_run = b->last_items;
  if (depths)
    for (int g = 0; g < b->n; g++) depths[g] = batch_depth(b->grids[g]);
  return 0;
}

}  // extern "C"
