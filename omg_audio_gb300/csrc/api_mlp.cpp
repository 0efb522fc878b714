// C ABI of the GB300 tracer (include/omg_cuda.h), part 4: the learned
// surrogate. An ensemble of MLPs (n_in -> hidden x n_hidden -> n_out, GELU)
// trained on the GPU with the tensor-core GEMM (mlp.cu): BF16 weights and
// activations, FP32 accumulation, FP32 master weights, AdamW with a cosine
// learning-rate decay, MSE on standardized targets. Inference returns the
// ensemble mean and spread in the caller's units.
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>

#include "runtime.h"

using namespace omg;

namespace omg {

struct MlpLayer {
  uint32_t in = 0, out = 0;
  DevBuf<float> W, b, mW, vW, mb, vb;
  float* gW = nullptr;    // the gradients: views into the member's gradient block
  float* gb = nullptr;
  DevBuf<uint16_t> Wh;    // bf16 copy of W [out x in]
  DevBuf<uint16_t> Wht;   // its transpose [in x out]: the K-major operand of dX = dZ . W
};

// The work buffers of one batch of `cap` rows. Besides the row-major
// activations and gradients, the backward pass keeps their bf16 transposes
// (xht, At, dZht: [features x rows]), so that every GEMM of training reads
// both operands K-major (the pipelined path of mlp.cu).
struct MlpBufs {
  uint32_t cap = 0;
  DevBuf<uint16_t> xh, xht;               // batch input (bf16) and its transpose
  DevBuf<float> t;                        // batch targets
  std::vector<DevBuf<float>> Z;           // pre-activations per layer
  std::vector<DevBuf<uint16_t>> A, At;    // bf16 activations per hidden layer, and transposes
  DevBuf<float> out, dX, dZ;
  DevBuf<uint16_t> dZh, dZht;
};

// One ensemble member's training lane: its buffers, stream, step graph,
// epoch permutation and device step counter.
struct MlpTrainer {
  MlpBufs bufs;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  DevBuf<uint32_t> perm, step;
  PinBuf<uint32_t> h_perm;
  PinBuf<float> h_loss;
  ~MlpTrainer() {
    if (graph) cudaGraphExecDestroy(graph);
    if (stream) cudaStreamDestroy(stream);
  }
};

struct MlpRec {
  omg_mlp_config cfg{};
  std::vector<std::vector<MlpLayer>> members;   // [member][layer]
  // per member, one block: every layer's gW then gb, then the loss (one memset clears it)
  std::vector<DevBuf<float>> grads;
  uint64_t grad_floats = 0;
  // standardization (host and device)
  std::vector<float> x_mean, x_std, y_mean, y_std;
  DevBuf<float> d_x_mean, d_x_std, d_y_mean, d_y_std;
  // inference buffers
  uint32_t icap = 0;
  DevBuf<float> xin, acc, acc2;
  PinBuf<float> h_x, h_mean, h_std;
  // dataset (standardized, device)
  uint32_t n_data = 0;
  DevBuf<float> X, Y;
  uint64_t step = 0;
  MlpBufs io;                                   // inference and omg_mlp_grad, on the context's stream
  std::vector<std::unique_ptr<MlpTrainer>> trainers;   // training, one per member
  DevBuf<float> sched;                          // per step: learning rate, bias corrections 1 and 2
  DevBuf<uint32_t> err;
  PinBuf<float> h_loss;
};

}  // namespace omg

namespace {

uint32_t n_layers(const MlpRec& M) { return M.cfg.n_hidden + 1; }

int32_t ensure_batch(omg_ctx* ctx, const MlpRec& M, MlpBufs& W, uint32_t rows, bool backward) {
  if (rows <= W.cap) return OMG_OK;
  const uint32_t L = n_layers(M), H = M.cfg.hidden;
  CK(W.xh.alloc((size_t)rows * M.cfg.n_in));
  CK(W.t.alloc((size_t)rows * M.cfg.n_out));
  W.Z.resize(L);
  W.A.resize(L);
  W.At.resize(L);
  for (uint32_t l = 0; l < L; l++) {
    const uint32_t o = l + 1 == L ? M.cfg.n_out : H;
    CK(W.Z[l].alloc((size_t)rows * o));
    CK(W.A[l].alloc((size_t)rows * o));
    if (backward) CK(W.At[l].alloc((size_t)rows * o));
  }
  const uint32_t wide = std::max(std::max(H, M.cfg.n_out), M.cfg.n_in);
  CK(W.out.alloc((size_t)rows * M.cfg.n_out));
  CK(W.dX.alloc((size_t)rows * wide));
  CK(W.dZ.alloc((size_t)rows * wide));
  CK(W.dZh.alloc((size_t)rows * wide));
  if (backward) {
    CK(W.xht.alloc((size_t)rows * M.cfg.n_in));
    CK(W.dZht.alloc((size_t)rows * wide));
  }
  W.cap = rows;
  return OMG_OK;
}

// columns per CTA of a GEMM with n output columns: 64 (more, smaller CTAs:
// these GEMMs are short and latency-bound), or all of them when fewer
uint32_t n_tile_of(uint32_t n) { return n > 64 ? 64u : ((n + 15) & ~15u); }

// X0 (bf16, rows x n_in) -> out (f32, rows x n_out); keeps Z and A (and, for
// training, the transposed activations At) for backward
int32_t forward(omg_ctx* ctx, MlpRec& M, MlpBufs& W, uint32_t e, uint32_t rows, bool keep_t, cudaStream_t s) {
  const uint32_t L = n_layers(M);
  auto& net = M.members[e];
  const uint16_t* x = W.xh.p;
  uint32_t in = M.cfg.n_in;
  for (uint32_t l = 0; l < L; l++) {
    MlpLayer& Ly = net[l];
    const bool last = l + 1 == L;
    GemmArgs g{};
    g.A = x;
    g.a_rs = in;
    g.a_ks = 1;
    g.B = Ly.Wh.p;
    g.b_rs = Ly.in;
    g.b_ks = 1;
    g.M = rows;
    g.N = Ly.out;
    g.K = in;
    g.n_tile = n_tile_of(Ly.out);
    g.bias = Ly.b.p;
    g.err = M.err.p;
    if (last) {
      g.D = W.out.p;
      g.ldd = Ly.out;
    } else {
      g.Z = W.Z[l].p;
      g.ldz = Ly.out;
      g.Y = W.A[l].p;
      g.ldy = Ly.out;
      if (keep_t) {
        g.Yt = W.At[l].p;
        g.ldyt = rows;
      }
      g.act = 1;
    }
    CK(launch_gemm(g, 1, s));
    x = W.A[l].p;
    in = Ly.out;
  }
  return OMG_OK;
}

// gradients of the MSE (targets in W.t) into the layers' gW, gb and the loss
// into the member's gradient block (all zeroed here first, in one memset).
// Every GEMM reads K-major operands: dW = dZ^T X from the transposes dZht and
// xht / At, dX = dZ W from dZh and Wht.
int32_t backward(omg_ctx* ctx, MlpRec& M, MlpBufs& W, uint32_t e, uint32_t rows, cudaStream_t s) {
  const uint32_t L = n_layers(M);
  auto& net = M.members[e];
  float* loss = M.grads[e].p + M.grad_floats - 1;
  CK(cudaMemsetAsync(M.grads[e].p, 0, M.grad_floats * 4, s));   // every gW, gb and the loss
  MlpLayer& top = net[L - 1];
  CK(launch_grad_tile(0, W.out.p, W.t.p, nullptr, rows, M.cfg.n_out, W.dZ.p, W.dZh.p, W.dZht.p, top.gb, loss, s));
  for (int l = (int)L - 1; l >= 0; l--) {
    MlpLayer& Ly = net[l];
    const uint16_t* xt = l == 0 ? W.xht.p : W.At[l - 1].p;
    // dW = dZ^T . X  (reduction over the batch, split over grid z; gW zeroed above)
    GemmArgs g{};
    g.A = W.dZht.p;
    g.a_rs = rows;
    g.a_ks = 1;
    g.B = xt;
    g.b_rs = rows;
    g.b_ks = 1;
    g.M = Ly.out;
    g.N = Ly.in;
    g.K = rows;
    g.n_tile = n_tile_of(Ly.in);
    g.D = Ly.gW;
    g.ldd = Ly.in;
    g.accumulate = 1;
    g.err = M.err.p;
    const uint32_t split = std::max(1u, std::min(8u, rows / 512u));
    CK(launch_gemm(g, split, s));
    if (l == 0) break;
    // dX = dZ . W, then dZ of the layer below through GELU' (and its bias gradient)
    GemmArgs h{};
    h.A = W.dZh.p;
    h.a_rs = Ly.out;
    h.a_ks = 1;
    h.B = Ly.Wht.p;
    h.b_rs = Ly.out;
    h.b_ks = 1;
    h.M = rows;
    h.N = Ly.in;
    h.K = Ly.out;
    h.n_tile = n_tile_of(Ly.in);
    h.D = W.dX.p;
    h.ldd = Ly.in;
    h.err = M.err.p;
    CK(launch_gemm(h, 1, s));
    CK(launch_grad_tile(1, W.dX.p, W.Z[l - 1].p, nullptr, rows, Ly.in, W.dZ.p, W.dZh.p, W.dZht.p,
                        net[l - 1].gb, nullptr, s));
  }
  return OMG_OK;
}

int32_t check_err(omg_ctx* ctx, MlpRec& M) {
  uint32_t e = 0;
  CK(cudaMemcpyAsync(&e, M.err.p, 4, cudaMemcpyDeviceToHost, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  if (e) {
    ctx->last_error = "surrogate GEMM: an mbarrier wait ran out";
    CK(cudaMemsetAsync(M.err.p, 0, 4, ctx->stream));
    return OMG_E_TIMEOUT;
  }
  return OMG_OK;
}

int32_t sync_norm(omg_ctx* ctx, MlpRec& M) {
  if (!M.d_x_mean.p) {
    CK(M.d_x_mean.alloc(M.cfg.n_in));
    CK(M.d_x_std.alloc(M.cfg.n_in));
    CK(M.d_y_mean.alloc(M.cfg.n_out));
    CK(M.d_y_std.alloc(M.cfg.n_out));
  }
  CK(cudaMemcpy(M.d_x_mean.p, M.x_mean.data(), M.cfg.n_in * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(M.d_x_std.p, M.x_std.data(), M.cfg.n_in * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(M.d_y_mean.p, M.y_mean.data(), M.cfg.n_out * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(M.d_y_std.p, M.y_std.data(), M.cfg.n_out * 4, cudaMemcpyHostToDevice));
  return OMG_OK;
}

bool valid_cfg(const omg_mlp_config& c) {
  return c.n_in >= 1 && c.n_in <= 1024 && c.hidden >= 16 && c.hidden <= 256 && c.hidden % 16 == 0 &&
         c.n_hidden >= 1 && c.n_hidden <= 16 && c.n_out >= 1 && c.n_out <= 256 && c.members >= 1 &&
         c.members <= 16;
}

}  // namespace

extern "C" {

int32_t omg_mlp_create(omg_ctx* ctx, const omg_mlp_config* cfg, uint32_t* id) {
  if (!ctx || !cfg || !id || !valid_cfg(*cfg)) return OMG_E_INVALID;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, cudaGetLastError(), "cudaSetDevice");
  CK(gemm_init());
  std::shared_ptr<MlpRec> M(new MlpRec());
  M->cfg = *cfg;
  const uint32_t L = cfg->n_hidden + 1;
  std::mt19937_64 rng(cfg->seed ? cfg->seed : 1u);
  M->members.resize(cfg->members);
  for (uint32_t e = 0; e < cfg->members; e++) {
    M->members[e].resize(L);
    uint32_t in = cfg->n_in;
    for (uint32_t l = 0; l < L; l++) {
      MlpLayer& Ly = M->members[e][l];
      Ly.in = in;
      Ly.out = l + 1 == L ? cfg->n_out : cfg->hidden;
      const size_t nw = (size_t)Ly.out * Ly.in;
      // He-style normal init (std sqrt(2 / fan_in)), zero biases
      std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / (float)Ly.in));
      std::vector<float> w(nw);
      for (auto& v : w) v = nd(rng);
      if (l + 1 == L)
        for (auto& v : w) v *= 0.5f;
      CK(Ly.W.alloc(nw));
      CK(Ly.Wh.alloc(nw));
      CK(Ly.Wht.alloc(nw));
      CK(Ly.mW.alloc(nw));
      CK(Ly.vW.alloc(nw));

      CK(Ly.b.alloc(Ly.out));
      CK(Ly.mb.alloc(Ly.out));
      CK(Ly.vb.alloc(Ly.out));

      CK(cudaMemcpy(Ly.W.p, w.data(), nw * 4, cudaMemcpyHostToDevice));
      CK(cudaMemset(Ly.mW.p, 0, nw * 4));
      CK(cudaMemset(Ly.vW.p, 0, nw * 4));
      CK(cudaMemset(Ly.b.p, 0, Ly.out * 4));
      CK(cudaMemset(Ly.mb.p, 0, Ly.out * 4));
      CK(cudaMemset(Ly.vb.p, 0, Ly.out * 4));
      CK(launch_to_bf16_t(Ly.W.p, Ly.out, Ly.in, Ly.Wh.p, Ly.Wht.p, ctx->stream));
      in = Ly.out;
    }
  }
  // the gradient blocks: per member every layer's gW then gb, then the loss
  {
    uint64_t n = 1;
    for (auto& Ly : M->members[0]) n += (uint64_t)Ly.out * Ly.in + Ly.out;
    M->grad_floats = n;
    M->grads.resize(cfg->members);
    for (uint32_t e = 0; e < cfg->members; e++) {
      CK(M->grads[e].alloc(n));
      uint64_t off = 0;
      for (auto& Ly : M->members[e]) {
        Ly.gW = M->grads[e].p + off;
        off += (uint64_t)Ly.out * Ly.in;
        Ly.gb = M->grads[e].p + off;
        off += Ly.out;
      }
    }
  }
  M->x_mean.assign(cfg->n_in, 0.0f);
  M->x_std.assign(cfg->n_in, 1.0f);
  M->y_mean.assign(cfg->n_out, 0.0f);
  M->y_std.assign(cfg->n_out, 1.0f);
  CK(M->h_loss.alloc(1));
  CK(M->err.alloc(1));
  CK(cudaMemsetAsync(M->err.p, 0, 4, ctx->stream));
  CK(cudaStreamSynchronize(ctx->stream));
  int32_t rc = sync_norm(ctx, *M);
  if (rc) return rc;
  *id = ctx->next_mlp++;
  ctx->mlps[*id] = M;
  return OMG_OK;
}

int32_t omg_mlp_destroy(omg_ctx* ctx, uint32_t id) {
  if (!ctx) return OMG_E_INVALID;
  auto it = ctx->mlps.find(id);
  if (it == ctx->mlps.end()) return OMG_E_NOT_FOUND;
  cudaStreamSynchronize(ctx->stream);
  ctx->mlps.erase(it);
  return OMG_OK;
}

int32_t omg_mlp_set_data(omg_ctx* ctx, uint32_t id, const float* x, const float* y, uint32_t n) {
  if (!ctx || !x || !y || n == 0) return OMG_E_INVALID;
  auto it = ctx->mlps.find(id);
  if (it == ctx->mlps.end()) return OMG_E_NOT_FOUND;
  MlpRec& M = *it->second;
  const uint32_t ni = M.cfg.n_in, no = M.cfg.n_out;
  // standardization from the data (FP64 sums)
  for (int which = 0; which < 2; which++) {
    const float* d = which ? y : x;
    const uint32_t c = which ? no : ni;
    std::vector<double> s(c, 0.0), q(c, 0.0);
    for (uint64_t i = 0; i < n; i++)
      for (uint32_t k = 0; k < c; k++) {
        const double v = d[i * c + k];
        if (!std::isfinite(v)) return OMG_E_INVALID;
        s[k] += v;
        q[k] += v * v;
      }
    std::vector<float>& mean = which ? M.y_mean : M.x_mean;
    std::vector<float>& sd = which ? M.y_std : M.x_std;
    for (uint32_t k = 0; k < c; k++) {
      const double m = s[k] / n, var = std::max(q[k] / n - m * m, 0.0);
      mean[k] = (float)m;
      sd[k] = (float)std::max(std::sqrt(var), 1e-6);
    }
  }
  std::vector<float> xs((size_t)n * ni), ys((size_t)n * no);
  for (uint64_t i = 0; i < n; i++) {
    for (uint32_t k = 0; k < ni; k++) xs[i * ni + k] = (x[i * ni + k] - M.x_mean[k]) / M.x_std[k];
    for (uint32_t k = 0; k < no; k++) ys[i * no + k] = (y[i * no + k] - M.y_mean[k]) / M.y_std[k];
  }
  int32_t rc = sync_norm(ctx, M);
  if (rc) return rc;
  CK(M.X.alloc(xs.size()));
  CK(M.Y.alloc(ys.size()));
  CK(cudaMemcpy(M.X.p, xs.data(), xs.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(M.Y.p, ys.data(), ys.size() * 4, cudaMemcpyHostToDevice));
  M.n_data = n;
  return OMG_OK;
}

// Training. Every member trains on its own stream, concurrently: one step
// (gather the batch, forward, backward, AdamW of every layer, step counter) is
// recorded once into a CUDA graph per member and launched steps-per-epoch
// times per epoch; the step's batch rows (this epoch's permutation, uploaded
// before the epoch) and its learning rate and bias corrections (a schedule
// uploaded once) are read on the device at the step counter. The host waits
// once per epoch, for the losses.
int32_t omg_mlp_train(omg_ctx* ctx, uint32_t id, const omg_mlp_train_config* tc, float* epoch_loss) {
  if (!ctx || !tc || tc->epochs == 0 || tc->batch == 0 || tc->batch % 128 != 0) return OMG_E_INVALID;
  auto it = ctx->mlps.find(id);
  if (it == ctx->mlps.end()) return OMG_E_NOT_FOUND;
  MlpRec& M = *it->second;
  if (M.n_data < tc->batch) return OMG_E_INVALID;
  const uint32_t L = n_layers(M), B = tc->batch, E = M.cfg.members;
  const uint32_t spe = M.n_data / B;
  const uint64_t total = (uint64_t)spe * tc->epochs;
  if (total >= (1ull << 31)) return OMG_E_INVALID;
  // the schedule: cosine decay from lr to lr_final, AdamW bias corrections
  std::vector<float> sched(3 * total);
  for (uint64_t t = 0; t < total; t++) {
    const double prog = total > 1 ? (double)t / (double)(total - 1) : 1.0;
    sched[3 * t] = (float)(tc->lr_final + 0.5 * (tc->lr - tc->lr_final) * (1.0 + std::cos(3.14159265358979323846 * prog)));
    sched[3 * t + 1] = (float)(1.0 - std::pow((double)tc->beta1, (double)(t + 1)));
    sched[3 * t + 2] = (float)(1.0 - std::pow((double)tc->beta2, (double)(t + 1)));
  }
  CK(gemm_init());   // outside the captures below
  CK(M.sched.alloc(sched.size()));
  CK(cudaMemcpy(M.sched.p, sched.data(), sched.size() * 4, cudaMemcpyHostToDevice));
  CK(cudaStreamSynchronize(ctx->stream));
  M.trainers.resize(E);
  int32_t rc = OMG_OK;
  for (uint32_t e = 0; e < E; e++) {
    if (!M.trainers[e]) M.trainers[e].reset(new MlpTrainer());
    MlpTrainer& T = *M.trainers[e];
    if (!T.stream) CK(cudaStreamCreateWithFlags(&T.stream, cudaStreamNonBlocking));
    if ((rc = ensure_batch(ctx, M, T.bufs, B, true))) return rc;
    CK(T.perm.alloc(M.n_data));
    CK(T.h_perm.alloc(M.n_data));
    CK(T.step.alloc(1));
    CK(T.h_loss.alloc(1));
    CK(cudaMemsetAsync(T.step.p, 0, 4, T.stream));
    // record one training step
    if (T.graph) {
      cudaGraphExecDestroy(T.graph);
      T.graph = nullptr;
    }
    cudaStream_t s = T.stream;
    MlpBufs& W = T.bufs;
    CK(cudaStreamSynchronize(s));
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    auto record = [&]() -> int32_t {
      CK(launch_gather_pair(M.X.p, M.cfg.n_in, M.Y.p, M.cfg.n_out, T.perm.p, T.step.p, spe, B, W.xh.p, W.xht.p,
                            W.t.p, s));
      int32_t r;
      if ((r = forward(ctx, M, W, e, B, true, s))) return r;
      if ((r = backward(ctx, M, W, e, B, s))) return r;
      AdamwTable tab{};
      uint64_t off = 0;
      for (uint32_t l = 0; l < L; l++) {
        MlpLayer& Ly = M.members[e][l];
        tab.L[l] = AdamwLayer{Ly.W.p, Ly.mW.p, Ly.vW.p, Ly.b.p, Ly.mb.p, Ly.vb.p, Ly.gW, Ly.gb, Ly.Wh.p, Ly.Wht.p,
                              Ly.in, Ly.out, off};
        off += (uint64_t)Ly.in * Ly.out + Ly.out;
      }
      tab.n = L;
      tab.total = off;
      CK(launch_adamw_all(tab, M.sched.p, T.step.p, tc->beta1, tc->beta2, tc->eps, tc->weight_decay, s));
      CK(launch_step(T.step.p, s));
      return OMG_OK;
    };
    rc = record();
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (ce != cudaSuccess) return fail(ctx, ce, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(&T.graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return fail(ctx, ce, "cudaGraphInstantiate");
  }
  std::vector<std::mt19937_64> rngs;
  for (uint32_t e = 0; e < E; e++) rngs.emplace_back((tc->seed ? tc->seed : 7u) + 0x9E3779B97F4A7C15ull * e);
  for (uint32_t ep = 0; ep < tc->epochs; ep++) {
    for (uint32_t e = 0; e < E; e++) {
      MlpTrainer& T = *M.trainers[e];
      std::iota(T.h_perm.p, T.h_perm.p + M.n_data, 0u);
      std::shuffle(T.h_perm.p, T.h_perm.p + M.n_data, rngs[e]);
      CK(cudaMemcpyAsync(T.perm.p, T.h_perm.p, (size_t)M.n_data * 4, cudaMemcpyHostToDevice, T.stream));
    }
    for (uint32_t st = 0; st < spe; st++)
      for (uint32_t e = 0; e < E; e++) CK(cudaGraphLaunch(M.trainers[e]->graph, M.trainers[e]->stream));
    for (uint32_t e = 0; e < E; e++) {
      MlpTrainer& T = *M.trainers[e];
      CK(cudaMemcpyAsync(T.h_loss.p, M.grads[e].p + M.grad_floats - 1, 4, cudaMemcpyDeviceToHost, T.stream));
    }
    // the permutation buffers are refilled next epoch: wait for this one
    for (uint32_t e = 0; e < E; e++) {
      MlpTrainer& T = *M.trainers[e];
      CK(cudaStreamSynchronize(T.stream));
      if (epoch_loss) epoch_loss[(size_t)e * tc->epochs + ep] = T.h_loss.p[0];
    }
  }
  M.step += total;
  return check_err(ctx, M);
}

}  // extern "C"

namespace {

// Shared by omg_surrogate_predict and omg_surrogate_query: y_std (full
// spread) and/or row_spread (per row, the largest spread among outputs whose
// mean is >= level) are optional.
int32_t surrogate_run(omg_ctx* ctx, uint32_t id, const float* x, uint32_t n, float* y_mean, float* y_std,
                      float* row_spread, float level) {
  if (!ctx || !x || !y_mean || n == 0) return OMG_E_INVALID;
  auto it = ctx->mlps.find(id);
  if (it == ctx->mlps.end()) return OMG_E_NOT_FOUND;
  MlpRec& M = *it->second;
  const uint32_t ni = M.cfg.n_in, no = M.cfg.n_out, E = M.cfg.members;
  const uint32_t chunk = 32768;
  const uint32_t rows_max = std::min(n, chunk);
  int32_t rc = ensure_batch(ctx, M, M.io, rows_max, false);
  if (rc) return rc;
  if (M.icap < rows_max) {
    CK(M.xin.alloc((size_t)rows_max * ni));
    CK(M.acc.alloc((size_t)rows_max * no));
    CK(M.acc2.alloc((size_t)rows_max * no));
    CK(M.h_x.alloc((size_t)rows_max * ni));
    CK(M.h_mean.alloc((size_t)rows_max * no));
    CK(M.h_std.alloc((size_t)rows_max * no));
    M.icap = rows_max;
  }
  cudaStream_t s = ctx->stream;
  // everything on the device: standardize, every member's forward, the
  // ensemble's mean and spread in the targets' units
  for (uint32_t r0 = 0; r0 < n; r0 += chunk) {
    const uint32_t rows = std::min(chunk, n - r0);
    const uint64_t nx = (uint64_t)rows * ni, ny = (uint64_t)rows * no;
    std::memcpy(M.h_x.p, x + (uint64_t)r0 * ni, nx * 4);
    CK(cudaMemcpyAsync(M.xin.p, M.h_x.p, nx * 4, cudaMemcpyHostToDevice, s));
    CK(launch_standardize(M.xin.p, M.d_x_mean.p, M.d_x_std.p, ni, nx, M.io.xh.p, s));
    for (uint32_t e = 0; e < E; e++) {
      if ((rc = forward(ctx, M, M.io, e, rows, false, s))) return rc;
      CK(launch_ensemble(M.io.out.p, M.d_y_mean.p, M.d_y_std.p, no, ny, M.acc.p, M.acc2.p, e == 0, e + 1 == E,
                         1.0f / (float)E, s));
    }
    CK(cudaMemcpyAsync(M.h_mean.p, M.acc.p, ny * 4, cudaMemcpyDeviceToHost, s));
    if (y_std) CK(cudaMemcpyAsync(M.h_std.p, M.acc2.p, ny * 4, cudaMemcpyDeviceToHost, s));
    if (row_spread) {
      // the per-row spread reuses the bf16 input buffer's space as f32 scratch
      CK(launch_row_spread(M.acc.p, M.acc2.p, no, rows, level, M.xin.p, s));
      CK(cudaMemcpyAsync(row_spread + r0, M.xin.p, (size_t)rows * 4, cudaMemcpyDeviceToHost, s));
    }
    CK(cudaStreamSynchronize(s));
    std::memcpy(y_mean + (uint64_t)r0 * no, M.h_mean.p, ny * 4);
    if (y_std) std::memcpy(y_std + (uint64_t)r0 * no, M.h_std.p, ny * 4);
  }
  return check_err(ctx, M);
}

}  // namespace

extern "C" {

int32_t omg_surrogate_predict(omg_ctx* ctx, uint32_t id, const float* x, uint32_t n, float* y_mean, float* y_std) {
  return surrogate_run(ctx, id, x, n, y_mean, y_std, nullptr, 0.0f);
}

int32_t omg_surrogate_query(omg_ctx* ctx, uint32_t id, const float* x, uint32_t n, float* y_mean,
                            float* row_spread, float level) {
  if (!row_spread) return OMG_E_INVALID;
  return surrogate_run(ctx, id, x, n, y_mean, nullptr, row_spread, level);
}

// One forward/backward of `member` on standardized inputs and targets: the
// loss and the gradients of every layer (W row-major, then b), in order.
int32_t omg_mlp_grad(omg_ctx* ctx, uint32_t id, uint32_t member, const float* x, const float* y, uint32_t n,
                     float* loss, float* grads) {
  if (!ctx || !x || !y || n == 0 || n % 128 != 0) return OMG_E_INVALID;
  auto it = ctx->mlps.find(id);
  if (it == ctx->mlps.end()) return OMG_E_NOT_FOUND;
  MlpRec& M = *it->second;
  if (member >= M.cfg.members) return OMG_E_INVALID;
  // the inference buffers may have been sized without the transposes
  if (M.io.cap && !M.io.xht.p) M.io.cap = 0;
  int32_t rc = ensure_batch(ctx, M, M.io, n, true);
  if (rc) return rc;
  cudaStream_t s = ctx->stream;
  MlpBufs& W = M.io;
  DevBuf<float> xd;
  CK(xd.alloc((size_t)n * M.cfg.n_in));
  CK(cudaMemcpyAsync(xd.p, x, (size_t)n * M.cfg.n_in * 4, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(W.t.p, y, (size_t)n * M.cfg.n_out * 4, cudaMemcpyHostToDevice, s));
  CK(launch_to_bf16_t(xd.p, n, M.cfg.n_in, W.xh.p, W.xht.p, s));
  if ((rc = forward(ctx, M, W, member, n, true, s))) return rc;
  if ((rc = backward(ctx, M, W, member, n, s))) return rc;
  CK(cudaMemcpyAsync(M.h_loss.p, M.grads[member].p + M.grad_floats - 1, 4, cudaMemcpyDeviceToHost, s));
  size_t off = 0;
  for (auto& Ly : M.members[member]) {
    if (grads) {
      CK(cudaMemcpyAsync(grads + off, Ly.gW, (size_t)Ly.out * Ly.in * 4, cudaMemcpyDeviceToHost, s));
      off += (size_t)Ly.out * Ly.in;
      CK(cudaMemcpyAsync(grads + off, Ly.gb, (size_t)Ly.out * 4, cudaMemcpyDeviceToHost, s));
      off += Ly.out;
    }
  }
  CK(cudaStreamSynchronize(s));
  if (loss) {
    *loss = M.h_loss.p[0];
  }
  return check_err(ctx, M);
}

// Parameters: what = 1: standardization (x mean, x std, y mean, y std) then
// every member's layers (W row-major, b); what = 2: the AdamW moments (mW, vW,
// mb, vb per layer per member) then the step count. out = null: count only.
int32_t omg_mlp_params(omg_ctx* ctx, uint32_t id, uint32_t what, float* out, uint64_t* count) {
  if (!ctx || !count || (what != 1 && what != 2)) return OMG_E_INVALID;
  auto it = ctx->mlps.find(id);
  if (it == ctx->mlps.end()) return OMG_E_NOT_FOUND;
  MlpRec& M = *it->second;
  uint64_t n = 0;
  auto put_host = [&](const std::vector<float>& v) {
    if (out) std::copy(v.begin(), v.end(), out + n);
    n += v.size();
  };
  auto put_dev = [&](const float* p, size_t k) -> cudaError_t {
    if (out) {
      cudaError_t e = cudaMemcpy(out + n, p, k * 4, cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return e;
    }
    n += k;
    return cudaSuccess;
  };
  CK(cudaStreamSynchronize(ctx->stream));
  if (what == 1) {
    put_host(M.x_mean);
    put_host(M.x_std);
    put_host(M.y_mean);
    put_host(M.y_std);
    for (auto& net : M.members)
      for (auto& Ly : net) {
        CK(put_dev(Ly.W.p, (size_t)Ly.out * Ly.in));
        CK(put_dev(Ly.b.p, Ly.out));
      }
  } else {
    for (auto& net : M.members)
      for (auto& Ly : net) {
        CK(put_dev(Ly.mW.p, (size_t)Ly.out * Ly.in));
        CK(put_dev(Ly.vW.p, (size_t)Ly.out * Ly.in));
        CK(put_dev(Ly.mb.p, Ly.out));
        CK(put_dev(Ly.vb.p, Ly.out));
      }
    if (out) out[n] = (float)M.step;
    n += 1;
  }
  *count = n;
  return OMG_OK;
}

int32_t omg_mlp_set_params(omg_ctx* ctx, uint32_t id, uint32_t what, const float* in, uint64_t count) {
  if (!ctx || !in || (what != 1 && what != 2)) return OMG_E_INVALID;
  auto it = ctx->mlps.find(id);
  if (it == ctx->mlps.end()) return OMG_E_NOT_FOUND;
  MlpRec& M = *it->second;
  uint64_t need = 0;
  int32_t rc = omg_mlp_params(ctx, id, what, nullptr, &need);
  if (rc) return rc;
  if (count != need) return OMG_E_INVALID;
  uint64_t n = 0;
  auto get_host = [&](std::vector<float>& v) {
    std::copy(in + n, in + n + v.size(), v.begin());
    n += v.size();
  };
  auto get_dev = [&](float* p, size_t k) -> cudaError_t {
    cudaError_t e = cudaMemcpy(p, in + n, k * 4, cudaMemcpyHostToDevice);
    n += k;
    return e;
  };
  if (what == 1) {
    get_host(M.x_mean);
    get_host(M.x_std);
    get_host(M.y_mean);
    get_host(M.y_std);
    for (auto& net : M.members)
      for (auto& Ly : net) {
        CK(get_dev(Ly.W.p, (size_t)Ly.out * Ly.in));
        CK(get_dev(Ly.b.p, Ly.out));
        CK(launch_to_bf16_t(Ly.W.p, Ly.out, Ly.in, Ly.Wh.p, Ly.Wht.p, ctx->stream));
      }
    int32_t rc2 = sync_norm(ctx, M);
    if (rc2) return rc2;
  } else {
    for (auto& net : M.members)
      for (auto& Ly : net) {
        CK(get_dev(Ly.mW.p, (size_t)Ly.out * Ly.in));
        CK(get_dev(Ly.vW.p, (size_t)Ly.out * Ly.in));
        CK(get_dev(Ly.mb.p, Ly.out));
        CK(get_dev(Ly.vb.p, Ly.out));
      }
    M.step = (uint64_t)in[n];
  }
  CK(cudaStreamSynchronize(ctx->stream));
  return OMG_OK;
}

// Device time of the tensor-core GEMM at one shape, for the record: A [m x k]
// and B [n x k] bf16 (K-major), C f32 (atomically accumulated when k_split >
// 1), operands resident on the device; `reps` launches between two events on
// the context's stream after 3 untimed ones. *ms = mean per launch.
int32_t omg_tc_gemm_bench(omg_ctx* ctx, uint32_t m, uint32_t n, uint32_t k, uint32_t k_split, uint32_t reps,
                          float* ms) {
  if (!ctx || !ms || m == 0 || n == 0 || k == 0 || k % 8 != 0 || reps == 0 || k_split == 0 || k_split > 64)
    return OMG_E_INVALID;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, cudaGetLastError(), "cudaSetDevice");
  cudaStream_t s = ctx->stream;
  DevBuf<uint16_t> da, db;
  DevBuf<float> dc;
  DevBuf<uint32_t> err;
  CK(da.alloc((size_t)m * k));
  CK(db.alloc((size_t)n * k));
  CK(dc.alloc((size_t)m * n));
  CK(err.alloc(1));
  CK(cudaMemsetAsync(err.p, 0, 4, s));
  CK(cudaMemsetAsync(da.p, 0x3C, (size_t)m * k * 2, s));   // bf16 0x3C3C (about 0.0115) everywhere
  CK(cudaMemsetAsync(db.p, 0x3C, (size_t)n * k * 2, s));
  CK(cudaMemsetAsync(dc.p, 0, (size_t)m * n * 4, s));
  GemmArgs g{};
  g.A = da.p;
  g.a_rs = k;
  g.a_ks = 1;
  g.B = db.p;
  g.b_rs = k;
  g.b_ks = 1;
  g.M = m;
  g.N = n;
  g.K = k;
  g.n_tile = n > 128 ? 128u : ((n + 15) & ~15u);
  g.D = dc.p;
  g.ldd = n;
  g.accumulate = k_split > 1 ? 1u : 0u;
  g.err = err.p;
  for (int i = 0; i < 3; i++) CK(launch_gemm(g, k_split, s));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, s));
  for (uint32_t i = 0; i < reps; i++) CK(launch_gemm(g, k_split, s));
  CK(cudaEventRecord(e1, s));
  CK(cudaEventSynchronize(e1));
  float t = 0.0f;
  CK(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  uint32_t e = 0;
  CK(cudaMemcpy(&e, err.p, 4, cudaMemcpyDeviceToHost));
  if (e) {
    ctx->last_error = "tensor-core GEMM: an mbarrier wait ran out";
    return OMG_E_TIMEOUT;
  }
  *ms = t / (float)reps;
  return OMG_OK;
}

// The tensor-core GEMM alone: C[M x N] (f32) = A[M x K] . B[N x K]^T, A and B
// given as bf16 bit patterns in host memory (row-major, K contiguous).
int32_t omg_tc_gemm(omg_ctx* ctx, const uint16_t* a, const uint16_t* b, float* c, uint32_t m, uint32_t n,
                    uint32_t k) {
  if (!ctx || !a || !b || !c || m == 0 || n == 0 || k == 0) return OMG_E_INVALID;
  cudaStream_t s = ctx->stream;
  DevBuf<uint16_t> da, db;
  DevBuf<float> dc;
  DevBuf<uint32_t> err;
  CK(da.alloc((size_t)m * k));
  CK(db.alloc((size_t)n * k));
  CK(dc.alloc((size_t)m * n));
  CK(err.alloc(1));
  CK(cudaMemsetAsync(err.p, 0, 4, s));
  CK(cudaMemcpyAsync(da.p, a, (size_t)m * k * 2, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(db.p, b, (size_t)n * k * 2, cudaMemcpyHostToDevice, s));
  GemmArgs g{};
  g.A = da.p;
  g.a_rs = k;
  g.a_ks = 1;
  g.B = db.p;
  g.b_rs = k;
  g.b_ks = 1;
  g.M = m;
  g.N = n;
  g.K = k;
  g.n_tile = n <= 256 ? ((n + 15) & ~15u) : 256;
  g.D = dc.p;
  g.ldd = n;
  g.err = err.p;
  CK(launch_gemm(g, 1, s));
  uint32_t e = 0;
  CK(cudaMemcpyAsync(c, dc.p, (size_t)m * n * 4, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&e, err.p, 4, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (e) {
    ctx->last_error = "tensor-core GEMM: an mbarrier wait ran out";
    return OMG_E_TIMEOUT;
  }
  return OMG_OK;
}

}  // extern "C"
