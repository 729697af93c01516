// Batches of independent VMC problems advanced together (nqs_gpu_batch_*).
//
// Every instance has its own Hamiltonian, lattice, ansatz, sampler and
// workspaces; a batch step runs, for each instance, the derived-table rebuild,
// the Philox chains, the FP32 estimator (local energies + Jacobian), the energy
// statistics and ESS, the column means, the centring / TF32 split and the
// tensor-core Gram, then ONE cooperative launch that factors, inverts and
// refines the systems of all instances (each instance owns a range of CTAs with
// its own grid barrier), then per instance delta = O_c^T y / N_s (sample space)
// and the update.  The first step runs uncaptured and autotunes the split of
// the cooperative launch's CTAs between the instances (candidate splits timed
// with CUDA events on the Grams of that step); from the second step the whole
// sequence is one CUDA graph replayed per step, the samplers' move counters
// living in device memory so that each replay draws new random numbers.
#include <math.h>

#include "nqs_amp.cuh"

namespace nqs {

struct Sampler;
bool sampler_produce_dev(Sampler *sm, int n, uint64_t **d_out, unsigned long long *move_dev);
void sampler_host_advance(Sampler *sm, int n);
uint64_t sampler_move_counter(const Sampler *sm);
int sampler_chains(const Sampler *sm);
const unsigned long long *sampler_counts(const Sampler *sm);
bool sampler_fp32(const Sampler *sm);

struct BatchInst {
    nqs_config_t cfg{};
    int sx = 0, sy = 0;
    Ansatz *a = nullptr;
    Sampler *s = nullptr;
    nqs_log_amp_fn_t fn = nullptr;
    void *user = nullptr;
    DevAmp A{};
    DevHam H{};
    int Ns = 0, C = 0;
    long P = 0;
    DevBuf<double> E, Ei, eps, O, gm, scal, delta, y, part, es;
    DevBuf<unsigned long long> move;
    MixedSys *mx = nullptr;
    double *h = nullptr;      // pinned: scal[16], nrm[2]
    int *hs = nullptr;        // pinned: mixed status, error word
    unsigned long long *hc = nullptr;   // pinned: sampler counters (accepted, proposed)
    int fp64_fallback = 0, fp64_conv = 0;   // last step solved in FP64 after an FP32 breakdown
    ~BatchInst() {
        if (mx) mixed_sys_free(mx);
        if (h) cudaFreeHost(h);
        if (hs) cudaFreeHost(hs);
        if (hc) cudaFreeHost(hc);
    }
};

struct Batch {
    std::vector<BatchInst *> inst;
    MixedBatch *mb = nullptr;
    std::vector<int> ctas;
    int bd_from = 0;                     // systems of order >= bd_from use 128-wide diagonal blocks
    std::vector<double> tune_ms;
    cudaGraphExec_t exec = nullptr;
    long graph_kernels = 0;
    int steps = 0;
    long fallbacks = 0;                  // instance steps re-solved in FP64
    int sweeps = 5, passes = 3, space = 0;
    std::vector<cudaStream_t> side;      // instances' work forks onto these and joins the main stream
    std::vector<cudaEvent_t> join;
    cudaEvent_t fork = nullptr;
    ~Batch() {
        if (exec) cudaGraphExecDestroy(exec);
        for (cudaStream_t s : side) cudaStreamDestroy(s);
        for (cudaEvent_t e : join) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        if (mb) mixed_batch_free(mb);
        for (BatchInst *b : inst) delete b;
    }
};

// True when the mixed solve of an instance broke down: a non-positive FP32
// pivot, or a CG residual above the bound (nrm = |r|^2, |rhs|^2).
__host__ __device__ inline bool mixed_broken(int status, const double *nrm) {
    const double rel = nrm[1] > 0.0 ? sqrt(nrm[0] / nrm[1]) : 0.0;
    return status >= 0 || !(rel <= MIXED_RESID_MAX);
}

// theta -= lr delta and ||delta||^2, with delta = 0 when the instance's mixed
// solve broke down or its kernels reported an error (decided by one thread: the
// test's FP64 division and square root cost 16 cycles per warp instruction on this
// GPU's FP64 pipe).
__global__ void k_batch_apply(double *params, const double *__restrict__ delta, long P, double lr, double *scal,
                              const int *mstatus, const int *merr, const double *mnrm, int unconditional) {
    __shared__ double red[1024];
    __shared__ bool zero_s;
    if (threadIdx.x == 0) zero_s = !unconditional && (mixed_broken(mstatus[0], mnrm) || merr[0] != 0);
    __syncthreads();
    const bool zero = zero_s;
    double s = 0.0;
    for (long k = threadIdx.x; k < P; k += blockDim.x) {
        const double d = zero ? 0.0 : delta[k];
        params[k] += -lr * d;
        s += d * d;
    }
    red[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) scal[S_NORM2] = red[0];
}

bool enqueue_gated_apply(double *params, const double *delta, long P, double lr, double *scal, const int *mstatus,
                         const int *merr, const double *mnrm) {
    NQS_LAUNCH("apply_update");
    k_batch_apply<<<1, 1024, 0, ctx().stream>>>(params, delta, P, lr, scal, mstatus, merr, mnrm, 0);
    return NQS_CUDA(cudaGetLastError());
}

static bool enqueue_front(BatchInst &b, cudaStream_t st) {
    uint64_t *bits = nullptr;
    if (!ansatz_refresh_derived(b.a) || !sampler_produce_dev(b.s, b.Ns, &bits, b.move.p) ||
        !launch_local_estimator(b.A, b.H, bits, b.Ns, b.E.p, b.Ei.p, b.O.p, nullptr, 1, true) ||
        !enqueue_energy_stats(b.E.p, b.Ns, b.C, b.scal.p, b.eps.p, b.es.p) ||
        !enqueue_col_means(b.O.p, b.Ns, b.P, b.scal.p, b.gm.p, b.part.p))
        return false;
    mixed_sys_front(b.mx, st, true);
    return NQS_CUDA(cudaGetLastError());
}

static bool enqueue_back(BatchInst &b, cudaStream_t st) {
    if (!mixed_sys_param_space(b.mx) && !enqueue_col_dot(b.O.p, b.Ns, b.P, b.y.p, 1.0 / (double)b.Ns, b.delta.p))
        return false;
    {
        NQS_LAUNCH("apply_update");
        k_batch_apply<<<1, 1024, 0, st>>>(b.a->d_params.p, b.delta.p, b.P, b.cfg.learning_rate, b.scal.p,
                                          mixed_sys_status(b.mx), mixed_sys_err(b.mx), mixed_sys_nrm(b.mx), 0);
    }
    return NQS_CUDA(cudaMemcpyAsync(b.h, b.scal.p, 16 * sizeof(double), cudaMemcpyDeviceToHost, st)) &&
           NQS_CUDA(cudaMemcpyAsync(b.h + 16, mixed_sys_nrm(b.mx), 2 * sizeof(double), cudaMemcpyDeviceToHost, st)) &&
           NQS_CUDA(cudaMemcpyAsync(b.hs, mixed_sys_status(b.mx), sizeof(int), cudaMemcpyDeviceToHost, st)) &&
           NQS_CUDA(cudaMemcpyAsync(b.hs + 1, mixed_sys_err(b.mx), sizeof(int), cudaMemcpyDeviceToHost, st)) &&
           NQS_CUDA(cudaMemcpyAsync(b.hc, sampler_counts(b.s), 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                    st)) &&
           NQS_CUDA(cudaMemcpyAsync(b.a->h_params, b.a->d_params.p, sizeof(double) * b.P, cudaMemcpyDeviceToHost,
                                    st));
}

// Run `work(instance)` for every instance on the side streams (instance i on
// stream i mod S, the library's launches redirected there), forked from and
// joined back into the main stream: independent instances overlap, and in a
// captured sequence they become parallel branches of the graph.
template <typename F>
static bool fork_join(Batch &B, cudaStream_t main, F work) {
    Context &c = ctx();
    if (!NQS_CUDA(cudaEventRecord(B.fork, main))) return false;
    for (cudaStream_t s : B.side)
        if (!NQS_CUDA(cudaStreamWaitEvent(s, B.fork, 0))) return false;
    bool ok = true;
    for (size_t i = 0; i < B.inst.size() && ok; i++) {
        c.stream = B.side[i % B.side.size()];
        ok = work(*B.inst[i], c.stream);
    }
    c.stream = main;
    for (size_t k = 0; k < B.side.size(); k++)
        ok = ok && NQS_CUDA(cudaEventRecord(B.join[k], B.side[k])) &&
             NQS_CUDA(cudaStreamWaitEvent(main, B.join[k], 0));
    return ok;
}

// Candidate splits of the cooperative launch's CTAs between the instances:
// the same count for every instance (1, 2, 4, ...) and counts proportional to
// n_i^e for e = 1, 2, 3 (n_i the order of instance i's system: its factor is
// n^3 work on a chain of n / 128 diagonal blocks), within the co-resident limit.
static std::vector<std::vector<int>> cta_candidates(const Batch &B, int cap) {
    const int K = (int)B.inst.size();
    std::vector<std::vector<int>> c;
    for (int u = 1; u * K <= cap && u <= 32; u *= 2) c.push_back(std::vector<int>((size_t)K, u));
    for (int e = 1; e <= 3; e++) {
        std::vector<double> w((size_t)K);
        double tot = 0.0;
        for (int i = 0; i < K; i++) tot += (w[i] = pow((double)mixed_sys_order(B.inst[i]->mx), (double)e));
        std::vector<int> prop((size_t)K);
        int used = 0;
        for (int i = 0; i < K; i++) {
            prop[i] = (int)floor(w[i] / tot * (double)(cap - K)) + 1;
            used += prop[i];
        }
        if (used <= cap) c.push_back(prop);
    }
    return c;
}

// Autotune on the Grams of the first step: re-run each instance's Gram from
// its split operands and time the cooperative launch for every candidate CTA
// split and every tile shape of the factor (the diagonal block width: 128 from
// order 4096, from 2048, from 1024, else 64); keep the fastest (its launch, after
// a last Gram, is the step's solve).
static bool autotune(Batch &B, cudaStream_t st) {
    const int cap = mixed_batch_capacity();
    if (cap < (int)B.inst.size()) {
        set_error("batch of %d instances needs at least one co-resident CTA each (device holds %d)",
                  (int)B.inst.size(), cap);
        return false;
    }
    std::vector<MixedSys *> sys;
    for (BatchInst *b : B.inst) sys.push_back(b->mx);
    const std::vector<std::vector<int>> cand = cta_candidates(B, cap);
    const int bd_cand[3] = {mixed_bd_default(), 2048, 1024};
    cudaEvent_t e0, e1;
    if (!NQS_CUDA(cudaEventCreate(&e0)) || !NQS_CUDA(cudaEventCreate(&e1))) return false;
    double best = 1e300;
    int bi = -1, bb = 0;
    B.tune_ms.clear();
    for (size_t k = 0; k < cand.size() * 3; k++) {
        const size_t c = k % cand.size();
        const int t = (int)(k / cand.size());
        MixedBatch *mb = mixed_batch_create(sys.data(), (int)sys.size(), cand[c].data(), bd_cand[t]);
        if (!mb) {
            B.tune_ms.push_back(-1.0);
            continue;
        }
        if (k > 0)
            for (BatchInst *b : B.inst) mixed_sys_front(b->mx, st, false);
        float ms = 0.f;
        const bool ok = NQS_CUDA(cudaEventRecord(e0, st)) && mixed_batch_launch(mb, st) &&
                        NQS_CUDA(cudaEventRecord(e1, st)) && NQS_CUDA(cudaEventSynchronize(e1)) &&
                        NQS_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        mixed_batch_free(mb);
        if (!ok) break;
        B.tune_ms.push_back(ms);
        if (ms < best) {
            best = ms;
            bi = (int)c;
            bb = bd_cand[t];
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (bi < 0) return false;
    B.ctas = cand[bi];
    B.bd_from = bb;
    B.mb = mixed_batch_create(sys.data(), (int)sys.size(), B.ctas.data(), B.bd_from);
    if (!B.mb) return false;
    for (BatchInst *b : B.inst) mixed_sys_front(b->mx, st, false);
    return mixed_batch_launch(B.mb, st);
}

}  // namespace nqs

using namespace nqs;

struct nqs_gpu_batch {
    Batch b;
};

extern "C" {

nqs_gpu_batch_t *nqs_gpu_batch_create(const nqs_gpu_instance_t *in, int count) {
    clear_error();
    if (!in || count <= 0) {
        set_error("invalid arguments");
        return nullptr;
    }
    if (!ensure_context()) return nullptr;
    Context &c = ctx();
    cudaStream_t st = c.stream;
    nqs_gpu_batch_t *h = new nqs_gpu_batch_t();
    Batch &B = h->b;
    B.sweeps = c.opts.refine_sweeps;
    B.passes = c.opts.gram_passes;
    B.space = c.opts.mixed_space;
    const int nside = count < 8 ? count : 8;
    B.side.resize((size_t)nside, nullptr);
    B.join.resize((size_t)nside, nullptr);
    for (int k = 0; k < nside; k++)
        if (!NQS_CUDA(cudaStreamCreateWithFlags(&B.side[k], cudaStreamNonBlocking)) ||
            !NQS_CUDA(cudaEventCreateWithFlags(&B.join[k], cudaEventDisableTiming))) {
            delete h;
            return nullptr;
        }
    if (!NQS_CUDA(cudaEventCreateWithFlags(&B.fork, cudaEventDisableTiming))) {
        delete h;
        return nullptr;
    }
    for (int i = 0; i < count; i++) {
        BatchInst *b = new BatchInst();
        B.inst.push_back(b);
        if (!in[i].cfg || !in[i].ansatz || !in[i].sampler) {
            set_error("instance %d: cfg, ansatz and sampler are required", i);
            delete h;
            return nullptr;
        }
        b->cfg = *in[i].cfg;
        b->sx = in[i].size_x;
        b->sy = in[i].size_y;
        b->a = (Ansatz *)in[i].ansatz;
        b->s = (Sampler *)in[i].sampler;
        b->fn = in[i].log_amp ? in[i].log_amp : nqs_ansatz_log_amp;
        b->user = in[i].log_amp ? in[i].log_amp_user : (void *)b->a;
        Ansatz *base = nullptr;
        if (!hamiltonian_build(&b->cfg, b->sx, b->sy, &b->H) || !build_amp(b->fn, b->user, b->H.N, &b->A, &base)) {
            delete h;
            return nullptr;
        }
        if (base != b->a || !fp32_capable(b->A) || !sampler_fp32(b->s) ||
            nqs_sampler_num_sites((nqs_sampler_t *)b->s) != b->H.N) {
            set_error("instance %d: needs an RBM / cRBM program of its ansatz and a Philox sampler of the same "
                      "sites created in the MIXED mode with fp32_estimator = 1", i);
            delete h;
            return nullptr;
        }
        b->Ns = b->cfg.num_samples;
        b->C = sampler_chains(b->s);
        b->P = b->a->P;
        const uint64_t mv = sampler_move_counter(b->s);
        if (b->Ns <= 0 || !b->E.ensure(b->Ns) || !b->Ei.ensure(b->Ns) || !b->eps.ensure(b->Ns) ||
            !b->O.ensure((size_t)b->Ns * b->P) || !b->gm.ensure(b->P) || !b->scal.ensure(16) ||
            !b->delta.ensure(b->P) || !b->y.ensure(b->Ns) || !b->move.ensure(1) ||
            !b->part.ensure((size_t)col_stats_scratch(b->Ns, b->P)) ||
            !b->es.ensure(energy_scratch_doubles(b->Ns)) ||
            !NQS_CUDA(cudaMemset(b->es.p, 0, sizeof(double) * energy_scratch_doubles(b->Ns))) ||
            !NQS_CUDA(cudaMemcpy(b->move.p, &mv, sizeof(mv), cudaMemcpyHostToDevice)) ||
            !NQS_CUDA(cudaMallocHost(&b->h, 18 * sizeof(double))) ||
            !NQS_CUDA(cudaMallocHost(&b->hs, 2 * sizeof(int))) ||
            !NQS_CUDA(cudaMallocHost(&b->hc, 2 * sizeof(unsigned long long)))) {
            delete h;
            return nullptr;
        }
        b->mx = mixed_sys_create();
        if (!mixed_sys_prepare(b->mx, b->O.p, b->gm.p, b->eps.p, b->Ns, b->P, b->cfg.sr_diag_shift, B.sweeps, B.passes,
                               B.space, b->y.p, b->delta.p)) {
            delete h;
            return nullptr;
        }
    }
    if (!NQS_CUDA(cudaStreamSynchronize(st))) {
        delete h;
        return nullptr;
    }
    return h;
}

int nqs_gpu_batch_step(nqs_gpu_batch_t *h, nqs_sr_step_info_t *infos) {
    clear_error();
    if (!h) return -1;
    Batch &B = h->b;
    Context &c = ctx();
    cudaStream_t st = c.stream;
    for (BatchInst *b : B.inst)
        if (!ansatz_sync(b->a)) return -1;
    auto front = [](BatchInst &b, cudaStream_t s) { return enqueue_front(b, s); };
    auto back = [](BatchInst &b, cudaStream_t s) { return enqueue_back(b, s); };
    if (B.steps == 0 || c.profiling) {
        if (!fork_join(B, st, front)) return -1;
        if (B.steps == 0) {
            if (!autotune(B, st)) return -1;
        } else if (!mixed_batch_launch(B.mb, st)) {
            return -1;
        }
        if (!fork_join(B, st, back)) return -1;
    } else {
        if (!B.exec) {
            cudaGraph_t graph;
            const long l0 = c.launches;
            if (!NQS_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal))) return -1;
            bool ok = fork_join(B, st, front);
            ok = ok && mixed_batch_launch(B.mb, st);
            ok = ok && fork_join(B, st, back);
            const bool ended = NQS_CUDA(cudaStreamEndCapture(st, &graph));
            if (!ok || !ended) return -1;
            B.graph_kernels = c.launches - l0;
            c.launches = l0;
            const bool inst_ok = NQS_CUDA(cudaGraphInstantiate(&B.exec, graph, 0));
            cudaGraphDestroy(graph);
            if (!inst_ok) {
                B.exec = nullptr;
                return -1;
            }
        }
        if (!NQS_CUDA(cudaGraphLaunch(B.exec, st))) return -1;
        c.launches += B.graph_kernels;
    }
    if (!NQS_CUDA(cudaStreamSynchronize(st))) return -1;
    B.steps++;
    // An instance whose mixed solve broke down (a pivot <= 0, or a CG residual
    // above the bound) had its update held at zero inside the graph; solve it
    // again in FP64 on the same centred O and eps, as the single-system step does.
    for (size_t i = 0; i < B.inst.size(); i++) {
        BatchInst *b = B.inst[i];
        b->fp64_fallback = 0;
        if (!mixed_broken(b->hs[0], b->h + 16) || b->hs[1] != 0) continue;
        int conv = 0;
        if (minsr_fp64_delta(b->O.p, b->eps.p, b->Ns, b->P, b->cfg.sr_diag_shift, b->delta.p, &conv) != 0)
            return -1;
        k_batch_apply<<<1, 1024, 0, st>>>(b->a->d_params.p, b->delta.p, b->P, b->cfg.learning_rate, b->scal.p,
                                          mixed_sys_status(b->mx), mixed_sys_err(b->mx), mixed_sys_nrm(b->mx), 1);
        if (!NQS_CUDA(cudaMemcpyAsync(b->h + S_NORM2, b->scal.p + S_NORM2, sizeof(double), cudaMemcpyDeviceToHost,
                                      st)) ||
            !NQS_CUDA(cudaMemcpyAsync(b->a->h_params, b->a->d_params.p, sizeof(double) * b->P,
                                      cudaMemcpyDeviceToHost, st)) ||
            !NQS_CUDA(cudaStreamSynchronize(st)))
            return -1;
        b->fp64_fallback = 1;
        b->fp64_conv = conv;
        B.fallbacks++;
    }
    int failed = 0;
    for (size_t i = 0; i < B.inst.size(); i++) {
        BatchInst *b = B.inst[i];
        sampler_host_advance(b->s, b->Ns);
        memcpy(b->a->h_shadow, b->a->h_params, sizeof(double) * b->P);
        if (b->hs[1]) failed = (int)i + 1;
        if (infos) {
            nqs_sr_step_info_t &f = infos[i];
            f.mean_energy = b->h[S_EMEAN];
            f.variance_energy = b->h[S_ESQ] - b->h[S_EMEAN] * b->h[S_EMEAN];
            f.update_norm = sqrt(b->h[S_NORM2]) * b->cfg.learning_rate;
            f.acceptance_ratio = b->hc[1] ? (double)b->hc[0] / (double)b->hc[1] : 0.0;
            f.cg_iterations = 0;
            f.converged = b->fp64_fallback ? b->fp64_conv : (!mixed_broken(b->hs[0], b->h + 16) && b->hs[1] == 0);
        }
    }
    if (failed) {
        set_error("batch instance %d: %s", failed - 1,
                  B.inst[failed - 1]->hs[1] == 2 ? "grid barrier timed out" : "tensor-core Gram timed out");
        return -1;
    }
    return 0;
}

int nqs_gpu_batch_ctas(const nqs_gpu_batch_t *h, int *out) {
    if (!h || !out || h->b.ctas.empty()) return -1;
    for (size_t i = 0; i < h->b.ctas.size(); i++) out[i] = h->b.ctas[i];
    return 0;
}

int nqs_gpu_batch_block_widths(const nqs_gpu_batch_t *b, int *out_bd) {
    if (!b || !out_bd || b->b.ctas.empty()) return -1;
    for (size_t i = 0; i < b->b.inst.size(); i++)
        out_bd[i] = mixed_sys_order(b->b.inst[i]->mx) >= b->b.bd_from ? 128 : 64;
    return 0;
}

int nqs_gpu_batch_tune_ms(const nqs_gpu_batch_t *h, double *out, int cap) {
    if (!h || !out) return -1;
    const int n = (int)h->b.tune_ms.size() < cap ? (int)h->b.tune_ms.size() : cap;
    for (int i = 0; i < n; i++) out[i] = h->b.tune_ms[i];
    return n;
}

long nqs_gpu_batch_fallbacks(const nqs_gpu_batch_t *h) { return h ? h->b.fallbacks : -1; }

void nqs_gpu_batch_free(nqs_gpu_batch_t *h) { delete h; }

}  // extern "C"
