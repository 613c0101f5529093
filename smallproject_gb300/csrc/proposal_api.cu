// proposal_api.cu - C ABI of the learned candidate proposal (no reference counterpart):
// per-view network state, online training on the view's reservoirs, checkpoints.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "internal.hpp"
#include "proposal.hpp"
#include "view.hpp"

namespace vxr {

struct Proposal {
    prop::Dims d;
    prop::Layout L;
    vxr_proposal_desc desc{};
    float* params = nullptr;       // FP32 master
    float* grads = nullptr;
    float* m = nullptr;            // Adam moments
    float* v = nullptr;
    __nv_bfloat16* wbf = nullptr;  // W1 | W2 | W3 | W4 in BF16
    uint32_t* clOff = nullptr;     // cluster CSR
    uint32_t* clMembers = nullptr;
    uint32_t* lightCluster = nullptr;
    uint64_t clusterVersion = 0;
    uint2* cand = nullptr;         // [kMaxCand][pixels]
    uint32_t* pairRows = nullptr;  // pixels_per_eval = 2: the inference's table rows [pixels] and their count
    uint32_t* pairCount = nullptr;
    // training batch
    uint32_t B = 0;
    float4* samples = nullptr;
    uint32_t* target = nullptr;
    float* weight = nullptr;
    float* X = nullptr;
    float* H1 = nullptr;
    float* H2 = nullptr;
    float* H3 = nullptr;
    float* Z = nullptr;
    float* dA = nullptr;
    float* dB = nullptr;
    float* dX = nullptr;
    float* scal = nullptr;         // [loss, wsum]
    // fused tensor-core step (train.cu)
    bool fused = false;            // training on the tensor cores (else the FP32 layered trainer)
    uint32_t fusedB = 0;           // batch size the fused buffers hold
    uint4* frag = nullptr;         // weight-gradient operands as mma fragments
    float* partials = nullptr;     // [chunk][MLP parameters] gradient sums
    float* lossPart = nullptr;     // [CTA]
    float* wpart = nullptr;        // weight sums per wsum block
    bool encGradDirty = true;      // the hash-table gradient is not known to be zero
    uint32_t online = 0;           // training steps run by every rendered frame
    // the frame's training step past its gather runs on a side stream and overlaps the next
    // frame; the view stream joins it (proposal_join) before anything reads the parameters
    // it writes or writes the batch it reads. Frame training steps are numbered (gen);
    // step g signals joinEv[g & 1].
    cudaStream_t trainStream = nullptr;
    cudaEvent_t forkEv = nullptr;
    cudaEvent_t joinEv[2] = {nullptr, nullptr};
    bool trainPending[2] = {false, false};
    uint64_t gen = 0;
    // desc.training_lag = 1: step g ends by publishing its parameters into slot g & 1, and
    // a frame's inference reads the slot of the step two frames back (joining only that
    // one), so a step has the whole next frame to run in
    float* pubParams[2] = {nullptr, nullptr};
    __nv_bfloat16* pubWbf[2] = {nullptr, nullptr};
    bool testTimeout = false;      // test hook: the inference issues no MMA and its waits give up
    int step = 0;
    uint32_t gatherOffset = 0;
};

void destroy_proposal(Proposal* p) {
    if (!p) return;
    if (p->trainStream) {
        cudaStreamSynchronize(p->trainStream);
        cudaStreamDestroy(p->trainStream);
    }
    if (p->forkEv) cudaEventDestroy(p->forkEv);
    for (int i = 0; i < 2; i++) {
        if (p->joinEv[i]) cudaEventDestroy(p->joinEv[i]);
        cudaFree(p->pubParams[i]);
        cudaFree(p->pubWbf[i]);
    }
    void* bufs[] = {p->params, p->grads, p->m, p->v, p->wbf, p->clOff, p->clMembers, p->lightCluster, p->cand,
                    p->pairRows, p->pairCount,
                    p->samples, p->target, p->weight, p->X, p->H1, p->H2, p->H3, p->Z, p->dA, p->dB, p->dX, p->scal,
                    p->partials, p->lossPart, p->wpart, p->frag};
    for (void* b : bufs) cudaFree(b);
    delete p;
}

}  // namespace vxr

using vxr::set_error;
using vxr::check_view;

#define CUP(call, what)                                                                                   \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return set_error(VXR_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e_)); \
    } while (0)

namespace {

size_t weights_count(const vxr::prop::Dims& d) {
    return (size_t)d.H * vxr::prop::kIn + 2 * (size_t)d.H * d.H + (size_t)d.K * d.H;
}

// refresh the BF16 inference copy of W1..W4 from the FP32 master
void refresh_bf16(vxr::Proposal* p, cudaStream_t s) {
    using namespace vxr::prop;
    const vxr::prop::Layout& L = p->L;
    const vxr::prop::Dims& d = p->d;
    __nv_bfloat16* o = p->wbf;
    launch_to_bf16(p->params + L.W1, o, (size_t)d.H * kIn, s);
    o += (size_t)d.H * kIn;
    launch_to_bf16(p->params + L.W2, o, (size_t)d.H * d.H, s);
    o += (size_t)d.H * d.H;
    launch_to_bf16(p->params + L.W3, o, (size_t)d.H * d.H, s);
    o += (size_t)d.H * d.H;
    launch_to_bf16(p->params + L.W4, o, (size_t)d.K * d.H, s);
}

// copies the current parameters (FP32 master, BF16 weights) into published slot `slot`
// (training_lag = 1), or into both slots (slot < 0); nothing without published slots
void publish(vxr::Proposal* p, int slot, cudaStream_t s) {
    if (!p->pubParams[0]) return;
    for (int i = 0; i < 2; i++) {
        if (slot >= 0 && i != slot) continue;
        cudaMemcpyAsync(p->pubParams[i], p->params, p->L.total * sizeof(float), cudaMemcpyDeviceToDevice, s);
        cudaMemcpyAsync(p->pubWbf[i], p->wbf, weights_count(p->d) * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice, s);
    }
}

// cluster CSR (members sorted by cluster, then light index) from the world's clustering
int upload_clusters(vxr_view* v, vxr::Proposal* p) {
    const vxr::World& w = v->world->w;
    const uint32_t n = (uint32_t)w.lights.size();
    const uint32_t K = (uint32_t)p->d.K;
    if (w.clusterCount != K || w.lightCluster.size() != n)
        return set_error(VXR_E_STATE, "proposal: the world's clustering does not match (run vxr_world_cluster_lights with k = " +
                                          std::to_string(K) + " after the last light change)");
    std::vector<uint32_t> off(K + 1, 0), mem(n);
    for (uint32_t i = 0; i < n; i++) off[w.lightCluster[i] + 1]++;
    for (uint32_t c = 0; c < K; c++) off[c + 1] += off[c];
    std::vector<uint32_t> pos(off.begin(), off.end() - 1);
    for (uint32_t i = 0; i < n; i++) mem[pos[w.lightCluster[i]]++] = i;
    for (uint32_t c = 0; c < K; c++)
        if (off[c + 1] == off[c]) return set_error(VXR_E_STATE, "proposal: empty cluster " + std::to_string(c));
    cudaFree(p->clOff);
    cudaFree(p->clMembers);
    cudaFree(p->lightCluster);
    p->clOff = nullptr; p->clMembers = nullptr; p->lightCluster = nullptr;
    CUP(cudaMalloc(&p->clOff, (K + 1) * sizeof(uint32_t)), "cudaMalloc(cluster offsets)");
    CUP(cudaMalloc(&p->clMembers, std::max<uint32_t>(n, 1) * sizeof(uint32_t)), "cudaMalloc(cluster members)");
    CUP(cudaMalloc(&p->lightCluster, std::max<uint32_t>(n, 1) * sizeof(uint32_t)), "cudaMalloc(light clusters)");
    CUP(cudaMemcpy(p->clOff, off.data(), (K + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice), "upload clusters");
    if (n) {
        CUP(cudaMemcpy(p->clMembers, mem.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice), "upload clusters");
        CUP(cudaMemcpy(p->lightCluster, w.lightCluster.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice),
            "upload clusters");
    }
    p->clusterVersion = w.clusterVersion;
    return VXR_OK;
}

// batch inputs (samples, targets, weights) for B samples, plus the working buffers of
// the selected trainer: per-CTA sums (fused) or the layer activations (FP32)
int ensure_batch(vxr::Proposal* p, uint32_t B) {
    using vxr::prop::kIn;
    if (B > p->B) {
        void** bufs[] = {(void**)&p->samples, (void**)&p->target, (void**)&p->weight, (void**)&p->X, (void**)&p->H1,
                         (void**)&p->H2, (void**)&p->H3, (void**)&p->Z, (void**)&p->dA, (void**)&p->dB, (void**)&p->dX};
        for (void** b : bufs) { cudaFree(*b); *b = nullptr; }
        CUP(cudaMalloc(&p->samples, B * sizeof(float4)), "cudaMalloc(batch)");
        CUP(cudaMalloc(&p->target, B * sizeof(uint32_t)), "cudaMalloc(batch)");
        CUP(cudaMalloc(&p->weight, B * sizeof(float)), "cudaMalloc(batch)");
        p->B = B;
    }
    if (p->fused) {
        if (p->fusedB < p->B) {
            cudaFree(p->partials);
            cudaFree(p->frag);
            p->partials = nullptr;
            p->frag = nullptr;
            p->fusedB = 0;
            const size_t n = (size_t)vxr::prop::train_chunks(p->B) * vxr::prop::train_mlp_count(p->d);
            CUP(cudaMalloc(&p->partials, n * sizeof(float)), "cudaMalloc(gradient sums)");
            CUP(cudaMalloc(&p->frag, vxr::prop::train_frag_bytes(p->d, p->B)), "cudaMalloc(gradient operands)");
            p->fusedB = p->B;
        }
        if (!p->lossPart) {
            CUP(cudaMalloc(&p->lossPart, vxr::prop::train_max_ctas() * sizeof(float)), "cudaMalloc(loss sums)");
            CUP(cudaMalloc(&p->wpart, vxr::prop::train_wsum_blocks() * sizeof(float)), "cudaMalloc(weight sums)");
        }
    } else if (!p->X) {
        const size_t H = p->d.H, K = p->d.K, n = p->B;
        CUP(cudaMalloc(&p->X, n * kIn * sizeof(float)), "cudaMalloc(batch)");
        CUP(cudaMalloc(&p->H1, n * H * sizeof(float)), "cudaMalloc(batch)");
        CUP(cudaMalloc(&p->H2, n * H * sizeof(float)), "cudaMalloc(batch)");
        CUP(cudaMalloc(&p->H3, n * H * sizeof(float)), "cudaMalloc(batch)");
        CUP(cudaMalloc(&p->Z, n * K * sizeof(float)), "cudaMalloc(batch)");
        CUP(cudaMalloc(&p->dA, n * H * sizeof(float)), "cudaMalloc(batch)");
        CUP(cudaMalloc(&p->dB, n * H * sizeof(float)), "cudaMalloc(batch)");
        CUP(cudaMalloc(&p->dX, n * kIn * sizeof(float)), "cudaMalloc(batch)");
    }
    return VXR_OK;
}

void forward_backward(vxr::Proposal* p, uint32_t B, cudaStream_t s);

// One gradient evaluation on the batch in p->samples/target/weight with the fused
// tensor-core step; apply = 1 also takes the Adam step (and refreshes the BF16 weights),
// apply = 0 leaves the full gradient in p->grads. [loss, weight sum] land in p->scal.
int fused_step(vxr::Proposal* p, uint32_t B, bool apply, cudaStream_t s) {
    using namespace vxr::prop;
    if (p->encGradDirty) {
        CUP(cudaMemsetAsync(p->grads + p->L.enc, 0, (size_t)kLevels * p->L.tableSize * kFeat * sizeof(float), s),
            "clear gradient");
        p->encGradDirty = false;
    }
    launch_wsum(p->weight, B, p->wpart, s);
    TrainArgs a{};
    a.dims = p->d;
    a.L = p->L;
    a.params = p->params;
    a.wbf = p->wbf;
    a.samples = p->samples;
    a.target = p->target;
    a.weight = p->weight;
    a.wpart = p->wpart;
    a.nwpart = train_wsum_blocks();
    a.B = B;
    a.grads = p->grads;
    a.frag = p->frag;
    a.partials = p->partials;
    a.lossPart = p->lossPart;
    int nparts = 0, nloss = 0;
    CUP(launch_train(a, s, &nparts, &nloss), "proposal training step");
    if (apply) p->step++;
    ReduceArgs r{};
    r.partials = p->partials;
    r.nparts = nparts;
    r.nmlp = train_mlp_count(p->d);
    r.K = p->d.K;
    r.lossPart = p->lossPart;
    r.nloss = nloss;
    r.wpart = p->wpart;
    r.nwpart = train_wsum_blocks();
    r.grads = p->grads + p->L.W1;
    r.params = p->params + p->L.W1;
    r.m = p->m + p->L.W1;
    r.v = p->v + p->L.W1;
    r.wbf = p->wbf;
    r.apply = apply ? 1 : 0;
    r.lr = p->desc.learning_rate;
    r.b1 = 0.9f;
    r.b2 = 0.999f;
    r.eps = 1e-8f;
    r.c1 = apply ? 1.0f / (1.0f - powf(r.b1, (float)p->step)) : 1.0f;
    r.c2 = apply ? 1.0f / (1.0f - powf(r.b2, (float)p->step)) : 1.0f;
    r.scal = p->scal;
    launch_train_reduce(r, s);
    if (apply) {
        launch_adam_enc(p->params + p->L.enc, p->grads + p->L.enc, p->m + p->L.enc, p->v + p->L.enc, p->L.W1 - p->L.enc,
                        p->desc.learning_rate, p->step, s);
    } else {
        p->encGradDirty = true;   // the caller reads the gradient; the next step clears it
    }
    CUP(cudaGetLastError(), "proposal training step");
    return VXR_OK;
}

// one training step on a batch gathered from the view's current frame
// the frame's training batch (B samples of its final reservoirs), on the view stream
static void gather_frame(vxr_view* v, vxr::Proposal* p) {
    const uint32_t B = p->desc.batch;
    vxr::prop::GatherArgs ga{};
    ga.k = vxr::dev_frame(v->k);
    ga.vd = v->buf.vd[v->cur];
    ga.hits = v->buf.hits;
    ga.count = v->buf.counters;
    ga.hA = v->buf.hA;
    ga.lightCluster = p->lightCluster;
    ga.nlights = (uint32_t)v->world->w.dev->nl;
    ga.B = B;
    ga.offset = p->gatherOffset;
    ga.samples = p->samples;
    ga.target = p->target;
    ga.weight = p->weight;
    p->gatherOffset = p->gatherOffset * 1664525u + 1013904223u;
    vxr::prop::launch_gather(ga, v->stream);
}

// one training step on the gathered batch (forward, backward, Adam), on stream s
static int train_batch(vxr::Proposal* p, cudaStream_t s) {
    const uint32_t B = p->desc.batch;
    if (p->fused) return fused_step(p, B, true, s);
    forward_backward(p, B, s);
    p->encGradDirty = true;
    p->step++;
    vxr::prop::launch_adam(p->params, p->grads, p->m, p->v, p->L.total, p->desc.learning_rate, p->step, s);
    refresh_bf16(p, s);
    CUP(cudaGetLastError(), "proposal training");
    return VXR_OK;
}

int train_on_frame(vxr_view* v, vxr::Proposal* p) {
    gather_frame(v, p);
    return train_batch(p, v->stream);
}

// forward + backward of the weighted cross-entropy on the batch in p->samples/target/weight;
// gradients (zeroed first) in p->grads, [loss, weight sum] in p->scal
void forward_backward(vxr::Proposal* p, uint32_t B, cudaStream_t s) {
    using namespace vxr::prop;
    const Layout& L = p->L;
    const Dims& d = p->d;
    const int H = d.H, K = d.K;
    float* P = p->params;
    float* G = p->grads;
    cudaMemsetAsync(G, 0, L.total * sizeof(float), s);
    cudaMemsetAsync(p->scal, 0, 2 * sizeof(float), s);
    launch_encode(P, L, d, p->samples, B, p->X, s);
    auto fwd = [&](const float* in, int kin, size_t wo, size_t bo, float* out, int nout, int mode) {
        GemmArgs g{};
        g.A = in; g.sam = kin; g.sak = 1;
        g.B = P + wo; g.sbk = 1; g.sbn = kin;
        g.C = out; g.scm = nout; g.scn = 1;
        g.M = (int)B; g.N = nout; g.K = kin;
        g.bias = P + bo; g.mode = mode;
        launch_gemm(g, s);
    };
    fwd(p->X, kIn, L.W1, L.b1, p->H1, H, 1);
    fwd(p->H1, H, L.W2, L.b2, p->H2, H, 1);
    fwd(p->H2, H, L.W3, L.b3, p->H3, H, 1);
    fwd(p->H3, H, L.W4, L.b4, p->Z, K, 2);
    launch_sum(p->weight, B, p->scal + 1, s);
    launch_softmax_ce(p->Z, p->target, p->weight, B, K, p->scal + 1, p->scal, s);
    // dW (out x in) += dY^T X over the batch (split-K, atomic), db = column sums of dY
    auto wgrad = [&](const float* dY, int nout, const float* Xin, int kin, size_t wo, size_t bo) {
        GemmArgs g{};
        g.A = dY; g.sam = 1; g.sak = nout;
        g.B = Xin; g.sbk = kin; g.sbn = 1;
        g.C = G + wo; g.scm = kin; g.scn = 1;
        g.M = nout; g.N = kin; g.K = (int)B;
        g.mode = 4; g.kchunk = 128;
        launch_gemm(g, s);
        launch_colsum(dY, B, nout, G + bo, s);
    };
    // dX_in = dY W (masked by relu of the layer input when mask != null)
    auto dgrad = [&](const float* dY, int nout, size_t wo, int kin, float* dXin, const float* mask) {
        GemmArgs g{};
        g.A = dY; g.sam = nout; g.sak = 1;
        g.B = P + wo; g.sbk = kin; g.sbn = 1;
        g.C = dXin; g.scm = kin; g.scn = 1;
        g.M = (int)B; g.N = kin; g.K = nout;
        g.mask = mask; g.smm = kin; g.mode = mask ? 3 : 0;
        launch_gemm(g, s);
    };
    wgrad(p->Z, K, p->H3, H, L.W4, L.b4);
    dgrad(p->Z, K, L.W4, H, p->dA, p->H3);        // dH3
    wgrad(p->dA, H, p->H2, H, L.W3, L.b3);
    dgrad(p->dA, H, L.W3, H, p->dB, p->H2);       // dH2
    wgrad(p->dB, H, p->H1, H, L.W2, L.b2);
    dgrad(p->dB, H, L.W2, H, p->dA, p->H1);       // dH1
    wgrad(p->dA, H, p->X, kIn, L.W1, L.b1);
    dgrad(p->dA, H, L.W1, kIn, p->dX, nullptr);   // dX
    launch_encode_backward(d, L, p->samples, p->dX, B, G, s);
}

}  // namespace

namespace vxr {
void proposal_join(vxr_view* v);

// the online training steps of a rendered frame (after shading: the frame's final
// reservoirs): the gather on the view's stream, the rest on the proposal's side stream;
// nothing when the view samples uniformly
int proposal_frame_train(vxr_view* v) {
    Proposal* p = v->prop;
    if (!v->useProposal || !p || !p->online) return VXR_OK;
    proposal_join(v);
    if (p->clusterVersion != v->world->w.clusterVersion)
        if (int r = upload_clusters(v, p)) return r;
    if (int r = ensure_batch(p, p->desc.batch)) return r;
    if (!p->trainStream) {
        // training_lag = 1: the lowest priority (the frames' kernels take free SM slots
        // first; a step has the whole next frame to finish); else the view stream's (the
        // next frame's inference waits for the step)
        int least = 0, greatest = 0;
        CUP(cudaDeviceGetStreamPriorityRange(&least, &greatest), "cudaDeviceGetStreamPriorityRange");
        CUP(cudaStreamCreateWithPriority(&p->trainStream, cudaStreamNonBlocking, p->desc.training_lag ? least : greatest),
            "cudaStreamCreate(training)");
        CUP(cudaEventCreateWithFlags(&p->forkEv, cudaEventDisableTiming), "cudaEventCreate");
        for (int i = 0; i < 2; i++) CUP(cudaEventCreateWithFlags(&p->joinEv[i], cudaEventDisableTiming), "cudaEventCreate");
    }
    const int slot = (int)(p->gen & 1u);
    for (uint32_t i = 0; i < p->online; i++) {
        proposal_join(v);   // a previous step still reads the batch the gather overwrites
        gather_frame(v, p);
        CUP(cudaEventRecord(p->forkEv, v->stream), "cudaEventRecord");
        CUP(cudaStreamWaitEvent(p->trainStream, p->forkEv, 0), "cudaStreamWaitEvent");
        if (i == 0 && v->ktimerOn && v->ktimer) v->ktimer->mark(K_TRAIN, false, p->trainStream);
        if (int r = train_batch(p, p->trainStream)) return r;
        if (i + 1 == p->online) {
            publish(p, slot, p->trainStream);
            if (v->ktimerOn && v->ktimer) v->ktimer->mark(K_TRAIN, true, p->trainStream);
        }
        CUP(cudaEventRecord(p->joinEv[slot], p->trainStream), "cudaEventRecord");
        p->trainPending[slot] = true;
    }
    p->gen++;
    return VXR_OK;
}

// stream s (the view's, or the one running the candidate passes) waits for the frame
// training steps still running on the side stream (slot < 0: all of them; else the one
// that signals joinEv[slot]); work that s hands on to the view's stream by an event
// carries the wait with it
static void join_slot(vxr_view* v, int slot, cudaStream_t s) {
    Proposal* p = v->prop;
    if (!p) return;
    for (int i = 0; i < 2; i++) {
        if ((slot >= 0 && i != slot) || !p->trainPending[i]) continue;
        cudaStreamWaitEvent(s, p->joinEv[i], 0);
        p->trainPending[i] = false;
    }
}

void proposal_join(vxr_view* v) { join_slot(v, -1, v->stream); }

// the candidate stage's hook (nullptr when the view samples uniformly)
bool learned_hook(vxr_view* v, LearnedHook* h, cudaStream_t s) {
    Proposal* p = v->prop;
    // the inference reads the weights of the last training step, or with training_lag = 1
    // the published ones of the step before it (slot (gen - 2) & 1 = gen & 1)
    const bool lag = p && p->pubParams[0];
    const int slot = p ? (int)(p->gen & 1u) : 0;
    join_slot(v, lag ? slot : -1, s);
    if (!v->useProposal || !p) return false;
    h->infer = prop::InferArgs{};
    h->infer.dims = p->d;
    h->infer.L = p->L;
    h->infer.params = lag ? p->pubParams[slot] : p->params;
    h->infer.wbf = lag ? p->pubWbf[slot] : p->wbf;
    h->infer.waitLimit = p->testTimeout ? 64u : 0u;
    h->infer.skipMma = p->testTimeout ? 1u : 0u;
    h->rows = p->desc.pixels_per_eval > 1 ? p->pairRows : nullptr;
    h->rowCount = p->pairCount;
    h->group = p->desc.pixels_per_eval;
    h->pairDist = p->desc.share_distance;
    h->cand = p->cand;
    h->clOff = p->clOff;
    h->clMembers = p->clMembers;
    h->lightCluster = p->lightCluster;
    return true;
}
}  // namespace vxr

extern "C" {

int vxr_proposal_default_desc(vxr_proposal_desc* d) {
    VXR_CHECK_ARG(d, "vxr_proposal_default_desc: null desc");
    std::memset(d, 0, sizeof(*d));
    d->hidden = 64;
    d->table_log2 = 16;
    d->res0 = 32;
    d->res1 = 128;
    d->epsilon = 0.1f;
    d->learning_rate = 1e-3f;
    d->batch = 65536;
    d->seed = 1;
    d->pixels_per_eval = 1;
    d->share_distance = 2.0f;
    return VXR_OK;
}

int vxr_view_proposal_enable(vxr_view* v, const vxr_proposal_desc* desc) {
    if (int r = check_view(v, "vxr_view_proposal_enable")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    VXR_CHECK_ARG(desc, "vxr_view_proposal_enable: null desc");
    VXR_CHECK_ARG(desc->epsilon > 0.0f && desc->epsilon <= 1.0f, "vxr_view_proposal_enable: epsilon must be in (0, 1]");
    VXR_CHECK_ARG(desc->table_log2 >= 8 && desc->table_log2 <= 22, "vxr_view_proposal_enable: table_log2 in [8, 22]");
    VXR_CHECK_ARG(desc->batch >= 1 && desc->batch <= (1u << 22), "vxr_view_proposal_enable: batch in [1, 2^22]");
    VXR_CHECK_ARG(desc->inference <= 2, "vxr_view_proposal_enable: inference must be 0 (auto), 1 (mma.sync) or 2 (tcgen05)");
    VXR_CHECK_ARG(v->desc.num_candidates <= (uint32_t)vxr::prop::kMaxCand,
                  "vxr_view_proposal_enable: at most 32 candidates per pixel with the learned proposal");
    vxr::prop::Dims d;
    d.H = (int)desc->hidden;
    d.K = (int)v->world->w.clusterCount;
    d.tableLog2 = (int)desc->table_log2;
    d.res0 = (int)desc->res0;
    d.res1 = (int)desc->res1;
    d.eps = desc->epsilon;
    d.kernel = (int)desc->inference;
    VXR_CHECK_ARG(d.K > 0, "vxr_view_proposal_enable: cluster the world's lights first (vxr_world_cluster_lights)");
    if (!vxr::prop::infer_supported(d))
        return set_error(VXR_E_INVALID, "vxr_view_proposal_enable: supported shapes are hidden = 64 and 16 <= clusters <= 1024, "
                                        "clusters a multiple of 16");
    if (d.kernel == 2 && !vxr::prop::infer_tc_supported(d))
        return set_error(VXR_E_INVALID, "vxr_view_proposal_enable: the tcgen05 inference needs hidden = 64 and 256 clusters");
    VXR_CHECK_ARG(desc->training <= 2, "vxr_view_proposal_enable: training must be 0 (auto), 1 (FP32) or 2 (tensor cores)");
    VXR_CHECK_ARG(desc->pixels_per_eval == 1 || desc->pixels_per_eval == 2 || desc->pixels_per_eval == 4 ||
                      desc->pixels_per_eval == 8,
                  "vxr_view_proposal_enable: pixels_per_eval must be 1, 2, 4 or 8");
    VXR_CHECK_ARG(v->npx < (1ull << 29), "vxr_view_proposal_enable: at most 2^29 - 1 pixels per view");
    VXR_CHECK_ARG(desc->training_lag <= 1, "vxr_view_proposal_enable: training_lag must be 0 or 1");
    VXR_CHECK_ARG(desc->pixels_per_eval == 1 || (desc->share_distance >= 0.0f && desc->share_distance <= 1e30f),
                  "vxr_view_proposal_enable: share_distance must be finite and >= 0");
    if (desc->training == 2 && !vxr::prop::train_supported(d))
        return set_error(VXR_E_INVALID, "vxr_view_proposal_enable: the tensor-core training step needs hidden = 64 and "
                                        "16 <= clusters <= 256");
    if (v->prop) vxr::destroy_proposal(v->prop);
    vxr::Proposal* p = new (std::nothrow) vxr::Proposal();
    if (!p) return set_error(VXR_E_NOMEM, "vxr_view_proposal_enable: out of host memory");
    v->prop = p;
    p->d = d;
    p->L = vxr::prop::layout(d);
    p->desc = *desc;
    p->fused = desc->training == 2 || (desc->training == 0 && vxr::prop::train_supported(d));
    const size_t n = p->L.total;
    CUP(cudaMalloc(&p->params, n * sizeof(float)), "cudaMalloc(params)");
    CUP(cudaMalloc(&p->grads, n * sizeof(float)), "cudaMalloc(grads)");
    CUP(cudaMalloc(&p->m, n * sizeof(float)), "cudaMalloc(adam)");
    CUP(cudaMalloc(&p->v, n * sizeof(float)), "cudaMalloc(adam)");
    CUP(cudaMalloc(&p->wbf, weights_count(d) * sizeof(__nv_bfloat16)), "cudaMalloc(bf16 weights)");
    CUP(cudaMalloc(&p->cand, v->npx * vxr::prop::kMaxCand * sizeof(uint2)), "cudaMalloc(candidates)");
    CUP(cudaMalloc(&p->scal, 2 * sizeof(float)), "cudaMalloc(scalars)");
    if (desc->training_lag) {
        for (int i = 0; i < 2; i++) {
            CUP(cudaMalloc(&p->pubParams[i], n * sizeof(float)), "cudaMalloc(published params)");
            CUP(cudaMalloc(&p->pubWbf[i], weights_count(d) * sizeof(__nv_bfloat16)), "cudaMalloc(published weights)");
        }
    }
    if (desc->pixels_per_eval > 1) {
        CUP(cudaMalloc(&p->pairRows, v->npx * sizeof(uint32_t)), "cudaMalloc(pair rows)");
        CUP(cudaMalloc(&p->pairCount, sizeof(uint32_t)), "cudaMalloc(pair rows)");
    }
    CUP(cudaMemsetAsync(p->m, 0, n * sizeof(float), v->stream), "clear adam");
    CUP(cudaMemsetAsync(p->v, 0, n * sizeof(float), v->stream), "clear adam");
    vxr::prop::launch_init(p->params, p->L, d, desc->seed, v->stream);
    refresh_bf16(p, v->stream);
    publish(p, -1, v->stream);
    CUP(cudaGetLastError(), "proposal init");
    if (int r = upload_clusters(v, p)) return r;
    CUP(cudaStreamSynchronize(v->stream), "proposal init");
    return VXR_OK;
}

int vxr_view_proposal_use(vxr_view* v, int on) {
    if (int r = check_view(v, "vxr_view_proposal_use")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    if (on && !v->prop) return set_error(VXR_E_STATE, "vxr_view_proposal_use: enable the proposal first");
    if (on && v->prop->clusterVersion != v->world->w.clusterVersion)
        if (int r = upload_clusters(v, v->prop)) return r;
    v->useProposal = on != 0;
    return VXR_OK;
}

int vxr_view_proposal_train(vxr_view* v, uint32_t steps, float* loss) {
    if (int r = check_view(v, "vxr_view_proposal_train")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    vxr::Proposal* p = v->prop;
    if (!p) return set_error(VXR_E_STATE, "vxr_view_proposal_train: enable the proposal first");
    if (p->clusterVersion != v->world->w.clusterVersion)
        if (int r = upload_clusters(v, p)) return r;
    if (int r = ensure_batch(p, p->desc.batch)) return r;
    float last = 0.0f;
    for (uint32_t it = 0; it < steps; it++) {
        if (int r = train_on_frame(v, p)) return r;
        if (it + 1 == steps && loss) {
            float h[2];
            CUP(cudaMemcpyAsync(h, p->scal, sizeof(h), cudaMemcpyDeviceToHost, v->stream), "read loss");
            CUP(cudaStreamSynchronize(v->stream), "proposal training");
            last = h[0];
        }
    }
    publish(p, -1, v->stream);
    if (loss) *loss = last;
    return VXR_OK;
}

int vxr_view_proposal_online(vxr_view* v, uint32_t steps_per_frame) {
    if (int r = check_view(v, "vxr_view_proposal_online")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    if (!v->prop) return set_error(VXR_E_STATE, "vxr_view_proposal_online: enable the proposal first");
    VXR_CHECK_ARG(steps_per_frame <= 16, "vxr_view_proposal_online: at most 16 steps per frame");
    if (steps_per_frame)
        if (int r = ensure_batch(v->prop, v->prop->desc.batch)) return r;
    v->prop->online = steps_per_frame;
    return VXR_OK;
}

int vxr_view_proposal_test_timeout(vxr_view* v, int on) {
    if (int r = check_view(v, "vxr_view_proposal_test_timeout")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    if (!v->prop) return set_error(VXR_E_STATE, "vxr_view_proposal_test_timeout: enable the proposal first");
    v->prop->testTimeout = on != 0;
    return VXR_OK;
}

int vxr_view_proposal_read_candidates(vxr_view* v, uint32_t* nhits, uint32_t* hits, uint32_t* cand) {
    if (int r = check_view(v, "vxr_view_proposal_read_candidates")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    VXR_CHECK_ARG(nhits, "vxr_view_proposal_read_candidates: null nhits");
    vxr::Proposal* p = v->prop;
    if (!p) return set_error(VXR_E_STATE, "vxr_view_proposal_read_candidates: enable the proposal first");
    CUP(cudaStreamSynchronize(v->stream), "vxr_view_proposal_read_candidates");
    uint32_t n = 0;
    CUP(cudaMemcpy(&n, v->buf.counters + vxr::kCtrHits, sizeof(n), cudaMemcpyDeviceToHost), "read hit count");
    *nhits = n;
    if (hits && n) CUP(cudaMemcpy(hits, v->buf.hits, n * sizeof(uint32_t), cudaMemcpyDeviceToHost), "read hit list");
    if (cand && n) {
        const uint32_t K = std::min(v->k.numberOfCandidates, v->k.numberOfLights);
        for (uint32_t m = 0; m < K; m++)
            CUP(cudaMemcpy(cand + (size_t)m * n * 2, p->cand + (size_t)m * v->npx, n * sizeof(uint2), cudaMemcpyDeviceToHost),
                "read candidates");
    }
    return VXR_OK;
}

int vxr_view_proposal_rows(vxr_view* v, uint32_t* rows) {
    if (int r = check_view(v, "vxr_view_proposal_rows")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    VXR_CHECK_ARG(rows, "vxr_view_proposal_rows: null rows");
    vxr::Proposal* p = v->prop;
    if (!p) return set_error(VXR_E_STATE, "vxr_view_proposal_rows: enable the proposal first");
    CUP(cudaStreamSynchronize(v->stream), "vxr_view_proposal_rows");
    const uint32_t* src = p->desc.pixels_per_eval > 1 ? p->pairCount : v->buf.counters + vxr::kCtrHits;
    CUP(cudaMemcpy(rows, src, sizeof(uint32_t), cudaMemcpyDeviceToHost), "read evaluation count");
    return VXR_OK;
}

int vxr_view_proposal_param_count(vxr_view* v, uint64_t* n, uint32_t* clusters, uint32_t* hidden) {
    if (int r = check_view(v, "vxr_view_proposal_param_count")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    VXR_CHECK_ARG(n, "vxr_view_proposal_param_count: null output");
    if (!v->prop) return set_error(VXR_E_STATE, "vxr_view_proposal_param_count: enable the proposal first");
    *n = v->prop->L.total;
    if (clusters) *clusters = (uint32_t)v->prop->d.K;
    if (hidden) *hidden = (uint32_t)v->prop->d.H;
    return VXR_OK;
}

int vxr_view_proposal_get_params(vxr_view* v, float* out) {
    if (int r = check_view(v, "vxr_view_proposal_get_params")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    VXR_CHECK_ARG(out, "vxr_view_proposal_get_params: null output");
    if (!v->prop) return set_error(VXR_E_STATE, "vxr_view_proposal_get_params: enable the proposal first");
    CUP(cudaStreamSynchronize(v->stream), "sync");
    CUP(cudaMemcpy(out, v->prop->params, v->prop->L.total * sizeof(float), cudaMemcpyDeviceToHost), "read params");
    return VXR_OK;
}

int vxr_view_proposal_set_params(vxr_view* v, const float* in) {
    if (int r = check_view(v, "vxr_view_proposal_set_params")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    VXR_CHECK_ARG(in, "vxr_view_proposal_set_params: null input");
    if (!v->prop) return set_error(VXR_E_STATE, "vxr_view_proposal_set_params: enable the proposal first");
    CUP(cudaStreamSynchronize(v->stream), "sync");
    CUP(cudaMemcpy(v->prop->params, in, v->prop->L.total * sizeof(float), cudaMemcpyHostToDevice), "write params");
    refresh_bf16(v->prop, v->stream);
    publish(v->prop, -1, v->stream);
    CUP(cudaStreamSynchronize(v->stream), "sync");
    return VXR_OK;
}

int vxr_view_proposal_grad(vxr_view* v, uint32_t B, const float* samples, const uint32_t* target, const float* weight,
                           float* loss, float* grad) {
    if (int r = check_view(v, "vxr_view_proposal_grad")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    VXR_CHECK_ARG(B >= 1 && samples && target && weight && loss && grad, "vxr_view_proposal_grad: bad argument");
    vxr::Proposal* p = v->prop;
    if (!p) return set_error(VXR_E_STATE, "vxr_view_proposal_grad: enable the proposal first");
    for (uint32_t b = 0; b < B; b++)
        VXR_CHECK_ARG(target[b] < (uint32_t)p->d.K, "vxr_view_proposal_grad: target cluster out of range");
    if (int r = ensure_batch(p, B)) return r;
    CUP(cudaStreamSynchronize(v->stream), "sync");
    CUP(cudaMemcpy(p->samples, samples, B * sizeof(float4), cudaMemcpyHostToDevice), "upload samples");
    CUP(cudaMemcpy(p->target, target, B * sizeof(uint32_t), cudaMemcpyHostToDevice), "upload targets");
    CUP(cudaMemcpy(p->weight, weight, B * sizeof(float), cudaMemcpyHostToDevice), "upload weights");
    if (p->fused) {
        if (int r = fused_step(p, B, false, v->stream)) return r;
    } else {
        forward_backward(p, B, v->stream);
        p->encGradDirty = true;
    }
    CUP(cudaGetLastError(), "proposal gradient");
    float h[2];
    CUP(cudaMemcpyAsync(h, p->scal, sizeof(h), cudaMemcpyDeviceToHost, v->stream), "read loss");
    CUP(cudaStreamSynchronize(v->stream), "sync");
    *loss = h[0];
    CUP(cudaMemcpy(grad, p->grads, p->L.total * sizeof(float), cudaMemcpyDeviceToHost), "read gradients");
    return VXR_OK;
}

int vxr_view_proposal_probs(vxr_view* v, uint32_t n, const float* samples, float* probs) {
    if (int r = check_view(v, "vxr_view_proposal_probs")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    VXR_CHECK_ARG(n >= 1 && samples && probs, "vxr_view_proposal_probs: bad argument");
    vxr::Proposal* p = v->prop;
    if (!p) return set_error(VXR_E_STATE, "vxr_view_proposal_probs: enable the proposal first");
    float4* ds = nullptr;
    float* dp = nullptr;
    CUP(cudaMalloc(&ds, n * sizeof(float4)), "cudaMalloc");
    if (cudaMalloc(&dp, (size_t)n * p->d.K * sizeof(float)) != cudaSuccess) {
        cudaFree(ds);
        return set_error(VXR_E_NOMEM, "vxr_view_proposal_probs: cudaMalloc");
    }
    cudaMemcpy(ds, samples, n * sizeof(float4), cudaMemcpyHostToDevice);
    vxr::prop::InferArgs a{};
    a.dims = p->d;
    a.L = p->L;
    a.params = p->params;
    a.wbf = p->wbf;
    a.samples = ds;
    a.n = n;
    a.probs = dp;
    a.err = v->buf.err;
    cudaError_t e = vxr::prop::launch_infer(a, n, v->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(v->stream);
    uint32_t flags = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&flags, v->buf.err, sizeof(flags), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && (flags & 16u)) {
        cudaMemset(v->buf.err, 0, sizeof(uint32_t));
        cudaFree(ds);
        cudaFree(dp);
        return set_error(VXR_E_DEVICE, "vxr_view_proposal_probs: a tensor-core wait gave up");
    }
    if (e == cudaSuccess) e = cudaMemcpy(probs, dp, (size_t)n * p->d.K * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(ds);
    cudaFree(dp);
    if (e != cudaSuccess) return set_error(VXR_E_CUDA, std::string("vxr_view_proposal_probs: ") + cudaGetErrorString(e));
    return VXR_OK;
}

// checkpoint: magic, version, dims, step, params, Adam moments
int vxr_view_proposal_save(vxr_view* v, const char* path) {
    if (int r = check_view(v, "vxr_view_proposal_save")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    VXR_CHECK_ARG(path, "vxr_view_proposal_save: null path");
    vxr::Proposal* p = v->prop;
    if (!p) return set_error(VXR_E_STATE, "vxr_view_proposal_save: enable the proposal first");
    const size_t n = p->L.total;
    std::vector<float> buf(3 * n);
    CUP(cudaStreamSynchronize(v->stream), "sync");
    CUP(cudaMemcpy(buf.data(), p->params, n * sizeof(float), cudaMemcpyDeviceToHost), "read params");
    CUP(cudaMemcpy(buf.data() + n, p->m, n * sizeof(float), cudaMemcpyDeviceToHost), "read adam");
    CUP(cudaMemcpy(buf.data() + 2 * n, p->v, n * sizeof(float), cudaMemcpyDeviceToHost), "read adam");
    FILE* f = std::fopen(path, "wb");
    if (!f) return set_error(VXR_E_IO, std::string("vxr_view_proposal_save: cannot open ") + path);
    const uint32_t hdr[8] = {0x56585250u /* "VXRP" */, 1u, (uint32_t)p->d.H, (uint32_t)p->d.K, (uint32_t)p->d.tableLog2,
                             (uint32_t)p->d.res0, (uint32_t)p->d.res1, (uint32_t)p->step};
    bool ok = std::fwrite(hdr, sizeof(hdr), 1, f) == 1 && std::fwrite(&p->d.eps, sizeof(float), 1, f) == 1 &&
              std::fwrite(buf.data(), sizeof(float), buf.size(), f) == buf.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return set_error(VXR_E_IO, std::string("vxr_view_proposal_save: write failed: ") + path);
    return VXR_OK;
}

int vxr_view_proposal_load(vxr_view* v, const char* path) {
    if (int r = check_view(v, "vxr_view_proposal_load")) return r;
    v->spatialEvOk = false;   // the next frame starts after this call's work
    vxr::proposal_join(v);
    VXR_CHECK_ARG(path, "vxr_view_proposal_load: null path");
    vxr::Proposal* p = v->prop;
    if (!p) return set_error(VXR_E_STATE, "vxr_view_proposal_load: enable the proposal first (same shape)");
    FILE* f = std::fopen(path, "rb");
    if (!f) return set_error(VXR_E_IO, std::string("vxr_view_proposal_load: cannot open ") + path);
    uint32_t hdr[8];
    float eps = 0.0f;
    const size_t n = p->L.total;
    std::vector<float> buf(3 * n);
    const bool ok = std::fread(hdr, sizeof(hdr), 1, f) == 1 && std::fread(&eps, sizeof(float), 1, f) == 1 &&
                    hdr[0] == 0x56585250u && hdr[1] == 1u && hdr[2] == (uint32_t)p->d.H && hdr[3] == (uint32_t)p->d.K &&
                    hdr[4] == (uint32_t)p->d.tableLog2 && hdr[5] == (uint32_t)p->d.res0 && hdr[6] == (uint32_t)p->d.res1 &&
                    std::fread(buf.data(), sizeof(float), buf.size(), f) == buf.size();
    std::fclose(f);
    if (!ok) return set_error(VXR_E_IO, std::string("vxr_view_proposal_load: malformed or mismatched checkpoint: ") + path);
    CUP(cudaStreamSynchronize(v->stream), "sync");
    CUP(cudaMemcpy(p->params, buf.data(), n * sizeof(float), cudaMemcpyHostToDevice), "write params");
    CUP(cudaMemcpy(p->m, buf.data() + n, n * sizeof(float), cudaMemcpyHostToDevice), "write adam");
    CUP(cudaMemcpy(p->v, buf.data() + 2 * n, n * sizeof(float), cudaMemcpyHostToDevice), "write adam");
    p->step = (int)hdr[7];
    refresh_bf16(p, v->stream);
    publish(p, -1, v->stream);
    CUP(cudaStreamSynchronize(v->stream), "sync");
    return VXR_OK;
}

}  // extern "C"
