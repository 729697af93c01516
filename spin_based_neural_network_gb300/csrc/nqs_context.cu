// Process-wide context: device, stream, options, errors, per-kernel timing.
#include <stdarg.h>

#include "nqs_internal.cuh"

namespace nqs {

static thread_local char g_err[512] = "";
static thread_local nqs_gpu_step_stats_t g_stats{};

nqs_gpu_step_stats_t &step_stats() { return g_stats; }

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

void clear_error() { g_err[0] = 0; }

bool cuda_ok(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return true;
    set_error("CUDA error %s (%d) in %s", cudaGetErrorString(e), (int)e, what);
    return false;
}

static nqs_gpu_options_t default_options() {
    nqs_gpu_options_t o;
    memset(&o, 0, sizeof(o));
    o.num_chains = 1;
    o.rng = NQS_GPU_RNG_XORSHIFT_COMPAT;
    o.move = NQS_GPU_MOVE_SINGLE_FLIP;
    o.n_down = -1;
    o.square_pbc = 0;
    o.precision = NQS_GPU_PREC_FP64;
    o.refine_sweeps = 2;
    o.gram_passes = 3;
    o.mixed_space = NQS_GPU_SPACE_AUTO;
    return o;
}

Context &ctx() {
    static Context c;
    return c;
}

bool ensure_context() {
    Context &c = ctx();
    std::lock_guard<std::mutex> lk(c.mu);
    if (c.initialised) {
        if (!c.usable) set_error("no usable CUDA device");
        return c.usable;
    }
    c.initialised = true;
    c.opts = default_options();
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        set_error("no CUDA device visible: this library has no CPU path");
        return false;
    }
    cudaGetDevice(&c.device);
    cudaDeviceProp prop;
    if (!NQS_CUDA(cudaGetDeviceProperties(&prop, c.device))) return false;
    if (prop.major < 10) {
        set_error("device %s (sm_%d%d) is not a Blackwell part; built for sm_103a", prop.name,
                  prop.major, prop.minor);
        return false;
    }
    c.sm_count = prop.multiProcessorCount;
    if (!NQS_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking))) return false;
    c.usable = true;
    return true;
}

LaunchScope::LaunchScope(const char *name) {
    Context &c = ctx();
    c.launches++;
    on = c.profiling;
    if (on) {
        ev.name = name;
        cudaEventCreate(&ev.a);
        cudaEventCreate(&ev.b);
        cudaEventRecord(ev.a, c.stream);
    }
}

LaunchScope::~LaunchScope() {
    if (!on) return;
    Context &c = ctx();
    cudaEventRecord(ev.b, c.stream);
    c.prof_pending.push_back(ev);
}

static void prof_drain() {
    Context &c = ctx();
    if (c.prof_pending.empty()) return;
    cudaStreamSynchronize(c.stream);
    for (auto &e : c.prof_pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e.a, e.b);
        auto &slot = c.prof_done[e.name];
        slot.first += 1;
        slot.second += ms;
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    c.prof_pending.clear();
}

// ---------------------------------------------------------------- configurations

uint64_t pack_spins(const int *s, int N) {
    uint64_t b = 0;
    for (int i = 0; i < N; i++)
        if (s[i] < 0) b |= 1ull << i;
    return b;
}

// Spin packing runs on the GPU: the host only copies the caller's int array.
__global__ void k_pack_spins(const int *__restrict__ s, int B, int N, uint64_t *__restrict__ bits) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    uint64_t v = 0;
    const int *row = s + (size_t)b * N;
    for (int i = 0; i < N; i++)
        if (row[i] < 0) v |= 1ull << i;
    bits[b] = v;
}

__global__ void k_bits_to_spins(const uint64_t *__restrict__ bits, int B, int N, int *__restrict__ out) {
    long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)B * N) return;
    int b = (int)(t / N), i = (int)(t % N);
    out[t] = ((bits[b] >> i) & 1ull) ? -1 : 1;
}

static DevBuf<int> g_spin_stage;
static DevBuf<uint64_t> g_bits_stage;

bool upload_spins(const int *spins, int B, int N, uint64_t **d_bits) {
    if (N <= 0 || N > kMaxSites) {
        set_error("num_sites %d outside the supported range 1..%d", N, kMaxSites);
        return false;
    }
    Context &c = ctx();
    if (!g_spin_stage.ensure((size_t)B * N) || !g_bits_stage.ensure((size_t)B)) return false;
    if (!NQS_CUDA(cudaMemcpyAsync(g_spin_stage.p, spins, sizeof(int) * (size_t)B * N,
                                  cudaMemcpyHostToDevice, c.stream)))
        return false;
    {
        NQS_LAUNCH("pack_spins");
        k_pack_spins<<<(B + 127) / 128, 128, 0, c.stream>>>(g_spin_stage.p, B, N, g_bits_stage.p);
    }
    *d_bits = g_bits_stage.p;
    return NQS_CUDA(cudaGetLastError());
}

bool launch_bits_to_spins(const uint64_t *bits, int B, int N, int *out) {
    Context &c = ctx();
    long tot = (long)B * N;
    NQS_LAUNCH("bits_to_spins");
    k_bits_to_spins<<<(unsigned)((tot + 255) / 256), 256, 0, c.stream>>>(bits, B, N, out);
    return NQS_CUDA(cudaGetLastError());
}

}  // namespace nqs

using namespace nqs;

extern "C" {

nqs_gpu_options_t nqs_gpu_options_default(void) { return default_options(); }

int nqs_gpu_set_options(const nqs_gpu_options_t *o) {
    if (!o) return -1;
    if (!ensure_context()) return -1;
    if (o->num_chains <= 0 || (o->rng != NQS_GPU_RNG_XORSHIFT_COMPAT && o->rng != NQS_GPU_RNG_PHILOX) ||
        (o->move != NQS_GPU_MOVE_SINGLE_FLIP && o->move != NQS_GPU_MOVE_EXCHANGE) ||
        (o->move == NQS_GPU_MOVE_EXCHANGE && o->rng != NQS_GPU_RNG_PHILOX) ||
        (o->precision != NQS_GPU_PREC_FP64 && o->precision != NQS_GPU_PREC_MIXED) || o->refine_sweeps < 0 ||
        (o->gram_passes != 1 && o->gram_passes != 3) || o->mixed_space < NQS_GPU_SPACE_AUTO ||
        o->mixed_space > NQS_GPU_SPACE_PARAMETERS || o->fp64_space < 0 || o->fp64_space > NQS_GPU_SPACE_SMALLER) {
        set_error("invalid nqs_gpu_options_t");
        return -1;
    }
    ctx().opts = *o;
    return 0;
}

int nqs_gpu_get_options(nqs_gpu_options_t *o) {
    if (!o) return -1;
    if (!ensure_context()) {
        *o = default_options();
        return -1;
    }
    *o = ctx().opts;
    return 0;
}

const char *nqs_gpu_last_error(void) { return g_err; }

int nqs_gpu_device_info(char *name, int len, int *sm_count) {
    if (!ensure_context()) return -1;
    cudaDeviceProp prop;
    if (!NQS_CUDA(cudaGetDeviceProperties(&prop, ctx().device))) return -1;
    if (name && len > 0) {
        strncpy(name, prop.name, (size_t)len - 1);
        name[len - 1] = 0;
    }
    if (sm_count) *sm_count = prop.multiProcessorCount;
    return 0;
}

void *nqs_gpu_stream(void) {
    if (!ensure_context()) return nullptr;
    return (void *)ctx().stream;
}

int nqs_gpu_synchronize(void) {
    if (!ensure_context()) return -1;
    return NQS_CUDA(cudaStreamSynchronize(ctx().stream)) ? 0 : -1;
}

int nqs_gpu_last_step_stats(nqs_gpu_step_stats_t *out) {
    if (!out) return -1;
    *out = g_stats;
    return 0;
}

int nqs_gpu_profile_enable(int on) {
    if (!ensure_context()) return -1;
    ctx().profiling = on != 0;
    if (!on) prof_drain();
    return 0;
}

int nqs_gpu_profile_reset(void) {
    if (!ensure_context()) return -1;
    prof_drain();
    ctx().prof_done.clear();
    ctx().launches = 0;
    return 0;
}

int nqs_gpu_profile_read(int cap, char names[][48], int *counts, double *ms) {
    if (!ensure_context()) return -1;
    prof_drain();
    int k = 0;
    for (auto &kv : ctx().prof_done) {
        if (k >= cap) break;
        if (names) {
            strncpy(names[k], kv.first.c_str(), 47);
            names[k][47] = 0;
        }
        if (counts) counts[k] = (int)kv.second.first;
        if (ms) ms[k] = kv.second.second;
        k++;
    }
    return k;
}

long nqs_gpu_launch_count(void) { return ctx().launches; }

void *nqs_gpu_event_record(void) {
    if (!ensure_context()) return nullptr;
    cudaEvent_t e;
    if (!NQS_CUDA(cudaEventCreate(&e))) return nullptr;
    if (!NQS_CUDA(cudaEventRecord(e, ctx().stream))) {
        cudaEventDestroy(e);
        return nullptr;
    }
    return (void *)e;
}

double nqs_gpu_event_elapsed_ms(void *a, void *b) {
    if (!a || !b) return -1.0;
    if (!NQS_CUDA(cudaEventSynchronize((cudaEvent_t)b))) return -1.0;
    float ms = 0.f;
    if (!NQS_CUDA(cudaEventElapsedTime(&ms, (cudaEvent_t)a, (cudaEvent_t)b))) return -1.0;
    return (double)ms;
}

void nqs_gpu_event_destroy(void *e) {
    if (e) cudaEventDestroy((cudaEvent_t)e);
}

}  // extern "C"
