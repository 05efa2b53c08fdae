// gb_batch.cu -- host side of the batched 2-D transforms (kernels in
// gb_batch_kernels.cuh): batch construction, the per-stage launches, CUDA
// graph capture and the autotuner.
#include "gb_batch_kernels.cuh"

namespace gb {

struct FftGroup {
  int n0, n1, count;
  long long off;  // arena offset of the first grid of the group
  cufftHandle h;
};

struct Batch {
  std::vector<nfftf_plan *> plans;
  std::vector<BPlan> host_plans;
  BPlan *d_plans = nullptr;
  long long *d_grid_off = nullptr, *d_fhat_off = nullptr;
  BItem *d_items = nullptr;
  int nitems = 0;
  BItem *d_items_col = nullptr;  // items of the plans in column mode
  int nitems_col = 0;
  WinPoly *d_polys = nullptr;    // the plans' polynomial windows
  size_t smem_col = 0;
  int grid_ctas_col = 0;
  int *d_counter = nullptr;  // [0] B queue head, [1] B^T queue head, [2], [3] the same for column items
  float2 *arena = nullptr;
  long long arena_total = 0, fhat_total = 0;
  std::vector<FftGroup> ffts;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  size_t smem = 0;
  int grid_ctas = 0;
  long long total_nodes = 0;
  cudaEvent_t ev[8] = {};
};

static void check_fft_b(cufftResult r, const char *what)
{
  if (r != CUFFT_SUCCESS) fatal("batch cuFFT %s failed (cufftResult %d)", what, (int)r);
}

// (re)build the device tables from the plans' current node set-up
static void batch_tables(Batch *b)
{
  const int np = (int)b->plans.size();
  std::vector<BItem> items, items_col;
  std::vector<long long> goff(np), foff(np);
  std::vector<WinPoly> polys(np);
  b->total_nodes = 0;
  size_t smem = 0, smem_col = 0;
  if (b->d_polys) GB_CUDA(cudaFree(b->d_polys));
  GB_CUDA(cudaMalloc(&b->d_polys, sizeof(WinPoly) * std::max(np, 1)));
  for (int k = 0; k < np; ++k) {
    PlanViewF v;
    plan_view_f(b->plans[k], &v);
    if (v.g.d != 2 || v.direct || !v.tiled || v.group3 || !v.ready)
      fatal("batch: plan %d is not a 2-D tiled plan with nodes set up", k);
    if (v.g.w != 10 && v.g.w != 14) fatal("batch: plan %d has m=%d (batched kernels take m = 4 or 6)", k, v.g.m);
    BPlan &P = b->host_plans[k];
    // tpn 0 asks for the column kernels, which need the plan's nodes keyed by column
    const int tpn = (P.tpn == 0 && !v.col2) ? 1 : P.tpn;
    memset(&P, 0, sizeof(P));
    polys[k] = *v.poly;
    P.poly = b->d_polys + k;
    P.g = v.g;
    P.xs = v.xs;
    P.perm = v.perm;
    P.cphi = v.cphi;
    P.fhat_in = v.fhat;
    P.f_out = v.f;
    P.f_in = v.f;
    P.fhat_out = v.fhat;
    P.tpn = tpn;
    b->total_nodes += v.g.M;
    if (tpn == 0)
      smem_col = std::max({smem_col, v.g.w == 10 ? c2_smem_bytes<10>(true) : c2_smem_bytes<14>(true),
                           v.g.w == 10 ? c2_smem_bytes<10>(false) : c2_smem_bytes<14>(false)});
    else
      smem = std::max(smem, (size_t)v.g.ext[0] * v.g.ext[1] * sizeof(float2));
    std::vector<WorkItem> wi(v.nitems);
    if (v.nitems)
      GB_CUDA(cudaMemcpy(wi.data(), v.items, sizeof(WorkItem) * v.nitems, cudaMemcpyDeviceToHost));
    for (const WorkItem &w : wi) (tpn == 0 ? items_col : items).push_back(BItem{k, w.tile, w.start, w.end});
  }
  // grids of equal shape are contiguous in the arena, one batched FFT per shape
  std::map<std::pair<int, int>, std::vector<int>> shapes;
  for (int k = 0; k < np; ++k) shapes[{b->host_plans[k].g.n[0], b->host_plans[k].g.n[1]}].push_back(k);
  long long off = 0, fo = 0;
  for (int k = 0; k < np; ++k) {
    b->host_plans[k].fhat_off = fo;
    foff[k] = fo;
    fo += b->host_plans[k].g.N_total;
  }
  for (auto &fg : b->ffts) cufftDestroy(fg.h);
  b->ffts.clear();
  std::vector<std::pair<long long, int>> order;  // arena offset -> plan, for the pad kernel's search
  for (auto &s : shapes) {
    FftGroup fg;
    fg.n0 = s.first.first;
    fg.n1 = s.first.second;
    fg.count = (int)s.second.size();
    fg.off = off;
    for (int k : s.second) {
      b->host_plans[k].grid_off = off;
      order.push_back({off, k});
      off += (long long)fg.n0 * fg.n1;
    }
    b->ffts.push_back(fg);
  }
  b->arena_total = off;
  b->fhat_total = fo;
  // the pad kernel walks the arena: order plans there by their arena offset
  std::vector<BPlan> pad_plans(np);
  for (int i = 0; i < np; ++i) {
    pad_plans[i] = b->host_plans[order[i].second];
    goff[i] = order[i].first;
  }
  if (b->arena) GB_CUDA(cudaFree(b->arena));
  GB_CUDA(cudaMalloc(&b->arena, sizeof(float2) * std::max<long long>(off, 1)));
  for (int k = 0; k < np; ++k) b->host_plans[k].grid = b->arena + b->host_plans[k].grid_off;
  for (int i = 0; i < np; ++i) pad_plans[i].grid = b->arena + pad_plans[i].grid_off;
  for (auto &fg : b->ffts) {
    int n[2] = {fg.n0, fg.n1};
    const int dist = fg.n0 * fg.n1;
    check_fft_b(cufftPlanMany(&fg.h, 2, n, nullptr, 1, dist, nullptr, 1, dist, CUFFT_C2C, fg.count), "plan");
    check_fft_b(cufftSetStream(fg.h, b->stream), "stream");
  }
  // largest items first: the persistent kernels then end with small work
  auto larger = [](const BItem &a, const BItem &c) { return (a.end - a.start) > (c.end - c.start); };
  std::stable_sort(items.begin(), items.end(), larger);
  std::stable_sort(items_col.begin(), items_col.end(), larger);
  b->nitems = (int)items.size();
  b->nitems_col = (int)items_col.size();
  GB_CUDA(cudaMemcpy(b->d_polys, polys.data(), sizeof(WinPoly) * np, cudaMemcpyHostToDevice));
  if (b->d_plans) GB_CUDA(cudaFree(b->d_plans));
  if (b->d_items) GB_CUDA(cudaFree(b->d_items));
  if (b->d_items_col) GB_CUDA(cudaFree(b->d_items_col));
  GB_CUDA(cudaMalloc(&b->d_items_col, sizeof(BItem) * std::max(b->nitems_col, 1)));
  if (b->nitems_col)
    GB_CUDA(cudaMemcpy(b->d_items_col, items_col.data(), sizeof(BItem) * b->nitems_col, cudaMemcpyHostToDevice));
  if (b->d_grid_off) GB_CUDA(cudaFree(b->d_grid_off));
  if (b->d_fhat_off) GB_CUDA(cudaFree(b->d_fhat_off));
  // device table: [0, np) by plan index (B, B^T, crop), [np, 2np) in arena order (pad)
  GB_CUDA(cudaMalloc(&b->d_plans, sizeof(BPlan) * 2 * np));
  GB_CUDA(cudaMemcpy(b->d_plans, b->host_plans.data(), sizeof(BPlan) * np, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMemcpy(b->d_plans + np, pad_plans.data(), sizeof(BPlan) * np, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMalloc(&b->d_items, sizeof(BItem) * std::max(b->nitems, 1)));
  if (b->nitems)
    GB_CUDA(cudaMemcpy(b->d_items, items.data(), sizeof(BItem) * b->nitems, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMalloc(&b->d_grid_off, sizeof(long long) * np));
  GB_CUDA(cudaMemcpy(b->d_grid_off, goff.data(), sizeof(long long) * np, cudaMemcpyHostToDevice));
  GB_CUDA(cudaMalloc(&b->d_fhat_off, sizeof(long long) * np));
  GB_CUDA(cudaMemcpy(b->d_fhat_off, foff.data(), sizeof(long long) * np, cudaMemcpyHostToDevice));
  b->smem = smem;
  set_smem_limit((const void *)k_batch_b2, 96 * 1024);
  set_smem_limit((const void *)k_batch_bt2, 96 * 1024);
  int per_sm = 0;
  GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_bt2, BT_THREADS, smem));
  int dev = 0, sms = 0;
  GB_CUDA(cudaGetDevice(&dev));
  GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  b->grid_ctas = std::max(1, per_sm) * sms;
  b->smem_col = smem_col;
  b->grid_ctas_col = 0;
  if (b->nitems_col) {
    set_smem_limit((const void *)k_batch_b2c, smem_col);
    set_smem_limit((const void *)k_batch_bt2c, smem_col);
    int per_sm_c = 0, per_sm_c2 = 0;
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_c, k_batch_bt2c, C2_THREADS, smem_col));
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_c2, k_batch_b2c, C2_THREADS, smem_col));
    b->grid_ctas_col = std::max(1, std::min(per_sm_c, per_sm_c2)) * sms;
  }
  if (b->graph_exec) {
    cudaGraphExecDestroy(b->graph_exec);
    b->graph_exec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
}

// f = A f_hat for every plan (device buffers of the plans)
static void batch_trafo_enqueue(Batch *b)
{
  const int np = (int)b->plans.size();
  cudaStream_t s = b->stream;
  const long long tot = b->arena_total;
  k_batch_pad<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(b->d_plans + np, b->d_grid_off, np, tot, b->arena);
  GB_LAUNCHED("batch_pad");
  for (auto &fg : b->ffts)
    check_fft_b(cufftExecC2C(fg.h, (cufftComplex *)(b->arena + fg.off), (cufftComplex *)(b->arena + fg.off),
                             CUFFT_FORWARD),
                "exec");
  if (b->nitems) {
    GB_CUDA(cudaMemsetAsync(b->d_counter, 0, sizeof(int), s));
    k_batch_b2<<<b->grid_ctas, BT_THREADS, b->smem, s>>>(b->d_plans, b->d_items, b->nitems, b->d_counter);
    GB_LAUNCHED("batch_b2");
  }
  if (b->nitems_col) {
    GB_CUDA(cudaMemsetAsync(b->d_counter + 2, 0, sizeof(int), s));
    k_batch_b2c<<<b->grid_ctas_col, C2_THREADS, b->smem_col, s>>>(b->d_plans, b->d_items_col, b->nitems_col,
                                                                  b->d_counter + 2);
    GB_LAUNCHED("batch_b2c");
  }
}

// f_hat = A^H f for every plan
static void batch_adjoint_enqueue(Batch *b)
{
  const int np = (int)b->plans.size();
  cudaStream_t s = b->stream;
  GB_CUDA(cudaMemsetAsync(b->arena, 0, sizeof(float2) * b->arena_total, s));
  if (b->nitems) {
    GB_CUDA(cudaMemsetAsync(b->d_counter + 1, 0, sizeof(int), s));
    k_batch_bt2<<<b->grid_ctas, BT_THREADS, b->smem, s>>>(b->d_plans, b->d_items, b->nitems, b->d_counter + 1);
    GB_LAUNCHED("batch_bt2");
  }
  if (b->nitems_col) {
    GB_CUDA(cudaMemsetAsync(b->d_counter + 3, 0, sizeof(int), s));
    k_batch_bt2c<<<b->grid_ctas_col, C2_THREADS, b->smem_col, s>>>(b->d_plans, b->d_items_col, b->nitems_col,
                                                                   b->d_counter + 3);
    GB_LAUNCHED("batch_bt2c");
  }
  for (auto &fg : b->ffts)
    check_fft_b(cufftExecC2C(fg.h, (cufftComplex *)(b->arena + fg.off), (cufftComplex *)(b->arena + fg.off),
                             CUFFT_INVERSE),
                "exec");
  const long long tot = b->fhat_total;
  k_batch_crop<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(b->d_plans, b->d_fhat_off, np, tot, b->arena);
  GB_LAUNCHED("batch_crop");
}

// trafo + adjoint of every plan captured once as a CUDA graph
static void batch_capture(Batch *b)
{
  if (b->graph_exec) return;
  GB_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  batch_trafo_enqueue(b);
  batch_adjoint_enqueue(b);
  GB_CUDA(cudaStreamEndCapture(b->stream, &b->graph));
  GB_CUDA(cudaGraphInstantiate(&b->graph_exec, b->graph, 0));
}

// ------------------------------------------------------------ autotuner
// Per class of plans (m, sigma, node density) the tile edge T in {8, 16, 32}
// and the threads per node in {1, 4, 16}, or the column kernels on 32^2 tiles
// (T = 0, tpn = 0), with the shortest B + B^T time, measured on up to four
// plans of the class run as their own batch.
struct TuneKey {
  int w, sigma100, dens;
  bool operator<(const TuneKey &o) const
  {
    return w != o.w ? w < o.w : (sigma100 != o.sigma100 ? sigma100 < o.sigma100 : dens < o.dens);
  }
};
struct TuneVal {
  int T, tpn;
  float ms;
};
static std::map<TuneKey, TuneVal> g_tune;

static TuneKey tune_key(const PlanViewF &v)
{
  const double dens = (double)v.g.M / (double)v.g.n_total;
  TuneKey k;
  k.w = v.g.w;
  k.sigma100 = (int)std::lround(100.0 * v.g.n[0] / v.g.N[0]);
  k.dens = (int)std::floor(std::log2(std::max(dens, 1e-9)));
  return k;
}

static float time_b_pair(Batch *b, int reps)
{
  batch_trafo_enqueue(b);  // warm-up
  batch_adjoint_enqueue(b);
  GB_CUDA(cudaEventRecord(b->ev[0], b->stream));
  for (int r = 0; r < reps; ++r) {
    GB_CUDA(cudaMemsetAsync(b->d_counter, 0, 4 * sizeof(int), b->stream));
    k_batch_b2<<<b->grid_ctas, BT_THREADS, b->smem, b->stream>>>(b->d_plans, b->d_items, b->nitems, b->d_counter);
    GB_LAUNCHED("batch_b2");
    k_batch_bt2<<<b->grid_ctas, BT_THREADS, b->smem, b->stream>>>(b->d_plans, b->d_items, b->nitems,
                                                                  b->d_counter + 1);
    GB_LAUNCHED("batch_bt2");
    if (b->nitems_col) {
      k_batch_b2c<<<b->grid_ctas_col, C2_THREADS, b->smem_col, b->stream>>>(b->d_plans, b->d_items_col,
                                                                            b->nitems_col, b->d_counter + 2);
      GB_LAUNCHED("batch_b2c");
      k_batch_bt2c<<<b->grid_ctas_col, C2_THREADS, b->smem_col, b->stream>>>(b->d_plans, b->d_items_col,
                                                                             b->nitems_col, b->d_counter + 3);
      GB_LAUNCHED("batch_bt2c");
    }
  }
  GB_CUDA(cudaEventRecord(b->ev[1], b->stream));
  GB_CUDA(cudaEventSynchronize(b->ev[1]));
  float ms = 0;
  GB_CUDA(cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
  return ms / reps;
}

static Batch *batch_new(nfftf_plan **plans, int count)
{
  Batch *b = new Batch();
  b->plans.assign(plans, plans + count);
  b->host_plans.resize(count);
  for (auto &P : b->host_plans) P.tpn = 1;
  GB_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  GB_CUDA(cudaMalloc(&b->d_counter, 4 * sizeof(int)));
  for (int i = 0; i < 8; ++i) GB_CUDA(cudaEventCreate(&b->ev[i]));
  for (auto *p : b->plans) GB_CUDA(cudaStreamSynchronize((cudaStream_t)nfftf_gb_get_stream(p)));
  batch_tables(b);
  return b;
}

static void batch_free(Batch *b)
{
  if (!b) return;
  cudaStreamSynchronize(b->stream);
  if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto &fg : b->ffts) cufftDestroy(fg.h);
  cudaFree(b->d_plans);
  cudaFree(b->d_items);
  cudaFree(b->d_items_col);
  cudaFree(b->d_polys);
  cudaFree(b->d_grid_off);
  cudaFree(b->d_fhat_off);
  cudaFree(b->d_counter);
  cudaFree(b->arena);
  for (int i = 0; i < 8; ++i)
    if (b->ev[i]) cudaEventDestroy(b->ev[i]);
  cudaStreamDestroy(b->stream);
  delete b;
}

static int batch_autotune(Batch *b, int reps)
{
  const int np = (int)b->plans.size();
  std::map<TuneKey, std::vector<int>> classes;
  for (int k = 0; k < np; ++k) {
    PlanViewF v;
    plan_view_f(b->plans[k], &v);
    classes[tune_key(v)].push_back(k);
  }
  const int Ts[3] = {8, 16, 32}, tpns[3] = {1, 4, 16};
  for (auto &cl : classes) {
    auto hit = g_tune.find(cl.first);
    if (hit == g_tune.end()) {
      // the class's largest plans (up to four) as a sample
      std::vector<int> idx = cl.second;
      std::sort(idx.begin(), idx.end(), [&](int a, int c) {
        return b->plans[a]->M_total > b->plans[c]->M_total;
      });
      idx.resize(std::min<size_t>(idx.size(), 4));
      std::vector<nfftf_plan *> sample;
      for (int k : idx) sample.push_back(b->plans[k]);
      TuneVal best = {32, 1, 1e30f};
      for (int T : Ts) {
        for (auto *p : sample) plan_retile_f(p, T);
        Batch *t = batch_new(sample.data(), (int)sample.size());
        for (int tpn : tpns) {
          for (auto &P : t->host_plans) P.tpn = tpn;
          GB_CUDA(cudaMemcpy(t->d_plans, t->host_plans.data(), sizeof(BPlan) * sample.size(),
                             cudaMemcpyHostToDevice));
          const float ms = time_b_pair(t, reps);
          if (ms < best.ms) best = {T, tpn, ms};
        }
        batch_free(t);
      }
      // the column kernels on the plans' own 32^2 tiles keyed by column
      bool col_ok = true;
      for (auto *p : sample) {
        plan_retile_f(p, 0);
        PlanViewF v;
        plan_view_f(p, &v);
        col_ok = col_ok && v.col2;
      }
      if (col_ok) {
        Batch *t = batch_new(sample.data(), (int)sample.size());
        for (auto &P : t->host_plans) P.tpn = 0;
        batch_tables(t);
        const float ms = time_b_pair(t, reps);
        if (ms < best.ms) best = {0, 0, ms};
        batch_free(t);
      }
      hit = g_tune.insert({cl.first, best}).first;
    }
    for (int k : cl.second) {
      plan_retile_f(b->plans[k], hit->second.T);
      b->host_plans[k].tpn = hit->second.tpn;
    }
  }
  batch_tables(b);
  return (int)classes.size();
}

}  // namespace gb

using namespace gb;

extern "C" {

void *nfftf_gb_batch_create(nfftf_plan **plans, int count)
{
  if (count < 1 || !plans) {
    record_error("nfftf_gb_batch_create: no plans");
    return nullptr;
  }
  return batch_new(plans, count);
}

void nfftf_gb_batch_destroy(void *batch) { batch_free(reinterpret_cast<Batch *>(batch)); }

int nfftf_gb_batch_autotune(void *batch, int reps)
{
  return batch_autotune(reinterpret_cast<Batch *>(batch), reps > 0 ? reps : 3);
}

// mode: 0 = stream launches, 1 = CUDA graph (captured on first use).
// what: 1 = trafo, 2 = adjoint, 3 = both.  Synchronises before returning.
int nfftf_gb_batch_run(void *batch, int what, int mode)
{
  Batch *b = reinterpret_cast<Batch *>(batch);
  if (mode == 1) {
    if (what != 3) {
      record_error("nfftf_gb_batch_run: the graph holds trafo + adjoint (what = 3)");
      return -1;
    }
    batch_capture(b);
    GB_CUDA(cudaGraphLaunch(b->graph_exec, b->stream));
  } else {
    if (what & 1) batch_trafo_enqueue(b);
    if (what & 2) batch_adjoint_enqueue(b);
  }
  GB_CUDA(cudaStreamSynchronize(b->stream));
  return 0;
}

// time `reps` trafo + adjoint rounds of the whole batch (ms per round)
float nfftf_gb_batch_time(void *batch, int reps, int mode)
{
  Batch *b = reinterpret_cast<Batch *>(batch);
  if (mode == 1) batch_capture(b);
  GB_CUDA(cudaEventRecord(b->ev[2], b->stream));
  for (int r = 0; r < reps; ++r) {
    if (mode == 1) {
      GB_CUDA(cudaGraphLaunch(b->graph_exec, b->stream));
    } else {
      batch_trafo_enqueue(b);
      batch_adjoint_enqueue(b);
    }
  }
  GB_CUDA(cudaEventRecord(b->ev[3], b->stream));
  GB_CUDA(cudaEventSynchronize(b->ev[3]));
  float ms = 0;
  GB_CUDA(cudaEventElapsedTime(&ms, b->ev[2], b->ev[3]));
  return ms / (reps > 0 ? reps : 1);
}

long long nfftf_gb_batch_nodes(void *batch) { return reinterpret_cast<Batch *>(batch)->total_nodes; }
int nfftf_gb_batch_items(void *batch) { return reinterpret_cast<Batch *>(batch)->nitems; }

// chosen (T, tpn) of plan k (after autotuning)
int nfftf_gb_batch_set_config(void *batch, int k, int T, int tpn)
{
  Batch *b = reinterpret_cast<Batch *>(batch);
  if (!b || k < 0 || k >= (int)b->plans.size()) return -1;
  if (tpn == 0) {
    if (T != 32) return -1;
    plan_retile_f(b->plans[k], 0);
    PlanViewF v;
    plan_view_f(b->plans[k], &v);
    if (!v.col2) return -1;
  } else {
    if ((T != 8 && T != 16 && T != 32) || (tpn != 1 && tpn != 4 && tpn != 16)) return -1;
    plan_retile_f(b->plans[k], T);
  }
  b->host_plans[k].tpn = tpn;
  batch_tables(b);
  return 0;
}

int nfftf_gb_batch_plan_config(void *batch, int k, int *T, int *tpn)
{
  Batch *b = reinterpret_cast<Batch *>(batch);
  if (k < 0 || k >= (int)b->plans.size()) return -1;
  *T = b->host_plans[k].g.T[0];
  *tpn = b->host_plans[k].tpn;
  return 0;
}

}  // extern "C"
