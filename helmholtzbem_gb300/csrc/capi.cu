// C ABI implementation (include/hbem.h): handles, device memory, streams and the
// host-side orchestration of the GPU kernels; host root finders.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <random>
#include <vector>

#include "../../include/hbem.h"
#include "assemble.cuh"

namespace hbem {
cudaError_t launch_flags(const DevMesh& M, const SingularTask* tasks, int ntasks, uint8_t* flags, cudaStream_t st);
size_t singular_geo_bytes(int nc, int ntasks);
cudaError_t launch_singular_geo(const DevMesh& M, const SingularTask* tasks, int ntasks, double* geo,
                                cudaStream_t st);
cudaError_t launch_local(const DevMesh& M, const SingularTask* tasks, int ntasks, const Job* jobs, int njobs,
                         bool real_k, int d, cplx* loc, cudaStream_t st, int layout, int which, double* part);
int singular_parts(int ntasks, int njobs);
size_t singular_part_bytes(int ntasks, int njobs, int d, bool curved);
cudaError_t launch_gather_T(int N, int d, const cplx* loc, const double* Mmass, int nk, int sp, cplx* T,
                            cudaStream_t st);
cudaError_t launch_local_multi(const MultiMesh* meshes, const MultiJob* jobs, int njobs, const long long* gstart,
                               long long gblocks, const long long* sstart, long long sblocks, int max_nc, bool curved,
                               bool real_k, int d, cplx* loc, cudaStream_t st);
cudaError_t launch_gather_layers(int N, int d, int layers, const cplx* loc, int job, int sp, cplx* out,
                                 cudaStream_t st);
cudaError_t launch_gather_layers_sub(int N, int d, int layers, const cplx* loc, int job, int row, int rows, int col,
                                     int cols, int sp, cplx* out, cudaStream_t st);
cudaError_t launch_projection(int N, const double* id, const double* sb, const double* lr, cplx* T, int nmat,
                              cudaStream_t st);
cudaError_t launch_taylor_near(long long mat, const cplx* src, int nq, double h0, double h1, int d, cplx* dst,
                               cudaStream_t st);
cudaError_t launch_svd(int n, int nmat, int D, int which, const cplx* T, long long mat_stride, long long der_stride,
                       cplx* gA, cplx* gV, double* out, double* sig_all, int* status, cudaStream_t st);
cudaError_t launch_svd_mixed(int n, int nmat, int D, int which, const cplx* T, long long mat_stride,
                             long long der_stride, cplx* gA, cplx* gV, double* out, double* sig_all, int* status,
                             cudaStream_t st);
cudaError_t launch_hankel01(int n, const cplx* z, int complex_arg, cplx* h0, cplx* h1, cudaStream_t st);
bool rsvd_supported(int n, int s, int D);
size_t rsvd_work_bytes(int n, int nmat, int s, int D, int precision);
cudaError_t rsvd_batched(int n, int nmat, int s, int q, int D, int precision, int refine, const cplx* T,
                         long long mat_stride, long long der_stride, const cplx* R, double* out, int* status,
                         void* work, size_t work_bytes, cudaStream_t st, long long* launches);
cudaError_t lu_factor_batched(int n, int nmat, cplx* A, long long stride, int* piv, int* perm, int* info,
                              cudaStream_t st, long long* launches);
cudaError_t lu_factor_batched_f32(int n, int nmat, cplxf* A, long long stride, int* piv, int* perm, int* info,
                                  cudaStream_t st, long long* launches, int* tc_err);
cudaError_t lu_solve_batched(int n, int nmat, int trans, const cplx* LU, long long stride, const int* perm, int s,
                             cplx* X, long long xstride, cudaStream_t st);
cudaError_t lu_perm_from_piv(int n, int nmat, const int* piv, int* perm, cudaStream_t st);
bool lu_solve_supported(int n);
void lu_set_cluster_panels(int on);
void lu_set_tensor_cores(int on);
void mlp_set_tensor_cores(int on);
int lu_get_cluster_panels();
void svd_set_pair_max(int m);
int svd_get_pair_max();
int lu_get_tensor_cores();
int mlp_get_tensor_cores();
cudaError_t launch_cgemm_f32(int m, int n, int k, const cplxf* A, long long lda, long long sa, const cplxf* B,
                             long long ldb, long long sb, cplxf* C, long long ldc, long long sc, int nmat,
                             int use_tc, int* err, cudaStream_t st);
size_t svd_fast_smem_bytes(int n);
bool arnoldi_supported(int n, int count, int D);
size_t arnoldi_work_bytes(int n, int nmat, int count, int D);
cudaError_t arnoldi_batched(int n, int nmat, int count, int D, double tol, int maxit, unsigned long long seed,
                            const cplx* T, long long mat_stride, long long der_stride, double* out, void* work,
                            size_t work_bytes, int* status_host, int* iters_host, cudaStream_t st,
                            long long* launches);
cudaError_t launch_svd_fast(int n, int nmat, int D, const cplx* T, long long mat_stride, long long der_stride,
                            double* out, int* status, cudaStream_t st, cplxf* vpool = nullptr,
                            const int* warm_slot = nullptr, const int* out_slot = nullptr, cplx* uv = nullptr);
cudaError_t launch_sigma1_uv(int n, int nmat, const cplx* T1, long long mat_stride, const cplx* uv, const int* idx,
                             double* d1, cudaStream_t st);
}  // namespace hbem

using namespace hbem;

namespace {

thread_local std::string g_err;
int g_device = 0;
const double kMachEps = 2.220446049250313e-16;

// instrumentation: kernel launches issued, and CUDA-event timing of the
// panel-pair assembly launches on the stream they run on (atomic: entry points may
// be called from several host threads on different operators)
std::atomic<long long> g_launches{0};
int g_timing = 0;
std::mutex g_stats_mu;
double g_asm_ms = 0.;
// CUDA events bracketing timed assembly launches, resolved (synchronised) when the
// statistics are read, so that timing does not stall the streams
std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_asm_pending;

// take the elapsed times of the pending event pairs into g_asm_ms (g_stats_mu held)
void resolve_pending_locked() {
    for (auto& pr : g_asm_pending) {
        float ms = 0.f;
        if (cudaEventSynchronize(pr.second) == cudaSuccess && cudaEventElapsedTime(&ms, pr.first, pr.second) == cudaSuccess)
            g_asm_ms += ms;
        cudaEventDestroy(pr.first);
        cudaEventDestroy(pr.second);
    }
    g_asm_pending.clear();
}

// start / end of a timed assembly launch on stream st (no wait)
void timing_begin(cudaEvent_t* e0, cudaStream_t st) {
    *e0 = nullptr;
    if (cudaEventCreate(e0) == cudaSuccess) cudaEventRecord(*e0, st);
}
void timing_end(cudaEvent_t e0, cudaStream_t st) {
    cudaEvent_t e1 = nullptr;
    if (!e0 || cudaEventCreate(&e1) != cudaSuccess) return;
    cudaEventRecord(e1, st);
    std::lock_guard<std::mutex> lk(g_stats_mu);
    g_asm_pending.emplace_back(e0, e1);
}
std::atomic<long long> g_asm_launches{0};
std::atomic<long long> g_asm_points{0};   // quadrature points x media processed by timed launches
// the same split by derivative order and by kind: [d] general pairs, [3 + d] singular
// pairs whose point data came from the builder's table, [6 + d] singular pairs that
// computed it in the kernel
std::atomic<long long> g_asm_split[9];
std::atomic<int> g_svd_fast{1};   // dense sigma: FP32 Jacobi + FP64 refinement where it fits
// per host thread: set while a sweep redoes, with the polished kernel, matrices the
// fast kernel could not finish; other threads keep the process-wide setting
thread_local int t_svd_polished_only = 0;
std::atomic<int> g_svd_force_redo{0};   // test hook: every fast-kernel result goes through the fallback
inline bool svd_fast_on() { return g_svd_fast.load(std::memory_order_relaxed) && !t_svd_polished_only; }
int g_arnoldi_maxit = 1000;   // block iterations of hbem_arnoldi_sv_batch*
int g_plain_speculate = 1;    // plain search: speculative bisection points in small Newton rounds
int g_singular_split = 1;     // launches of few jobs: singular pairs split over several CTAs each
thread_local int t_split_hold = 0;   // per host thread: no split while other streams keep the GPU full
int g_plain_warm_start = 1;   // plain search: dense-kernel Jacobi warm-started from nearby V sets
int g_plain_async = 1;        // plain search: Newton candidates advance independently on their own streams
int g_plain_spec_async = 2;   // ... speculating while at most this many candidates are unfinished
int g_plain_spec_deep = 2;    // ... two bisection levels deep while at most this many are
int g_singular_table = 1;     // singular pairs read their k-independent point data from a table
const size_t kSingularTableMax = (size_t)256 << 20;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define HB_CK(x)                                                                                     \
    do {                                                                                             \
        cudaError_t e_ = (x);                                                                        \
        if (e_ != cudaSuccess) return fail(HBEM_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// growable device buffer; requests below 64 MiB grow to the next power of two so
// that batches of varying size (Newton rounds) do not reallocate every call
struct DBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap) return cudaSuccess;
        if (bytes < ((size_t)64 << 20)) {
            size_t r = 256;
            while (r < bytes) r <<= 1;
            bytes = r;
        }
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, bytes);
        if (e == cudaSuccess) cap = bytes;
        return e;
    }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

template <class T>
cudaError_t upload(DBuf& b, const std::vector<T>& v, cudaStream_t st) {
    cudaError_t e = b.ensure(std::max<size_t>(1, v.size() * sizeof(T)));
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

// ---------------------------------------------------------------- host quadrature

// Gauss-Legendre nodes/weights on [a, b]: Newton on the three-term recurrence for
// P_n from the Chebyshev-like initial guesses, nodes stored ascending
// (the rule of include/gauleg.hpp:35-79).
void gauss_legendre(double a, double b, int n, double* x, double* w) {
    const int half = (n + 1) / 2;
    const double mid = 0.5 * (a + b), len = 0.5 * (b - a);
    for (int i = 0; i < half; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), zold, pn = 0., dpn = 0.;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1., p1 = 0.;
            for (int k = 1; k <= n; ++k) {
                double pm = p1;
                p1 = p0;
                p0 = ((2. * k - 1.) * z * p1 - (k - 1.) * pm) / k;
            }
            pn = p0;
            dpn = n * (z * p0 - p1) / (z * z - 1.0);
            zold = z;
            z = zold - pn / dpn;
            if (std::fabs(z - zold) <= kMachEps) break;
        }
        x[i] = mid - len * z;
        x[n - 1 - i] = mid + len * z;
        double wi = 2. * len / ((1. - z * z) * dpn * dpn);
        w[i] = wi;
        w[n - 1 - i] = wi;
    }
}

// Graded composite rule on [0, 1]: levels [s^(l+1), s^l], s = (sqrt2 - 1)^2, with
// Gauss orders n, n-1, ..., 2 from the top level down; n(n+1)/2 - 1 nodes,
// ascending (include/gauleg.hpp:89-121).
void graded_composite(int n, double* x, double* w) {
    const int N = n * (n + 1) / 2 - 1;
    const double sigma = (std::sqrt(2.) - 1.) * (std::sqrt(2.) - 1.);
    double lo = sigma, hi = 1.;
    int pos = N - 1;
    std::vector<double> gx(n), gw(n);
    for (int q = n; q >= 2; --q) {
        gauss_legendre(0., 1., q, gx.data(), gw.data());
        for (int j = q - 1; j >= 0; --j, --pos) {
            w[pos] = (hi - lo) * gw[j];
            x[pos] = (hi - lo) * gx[j] + lo;
        }
        hi = lo;
        lo *= sigma;
    }
}

// ---------------------------------------------------------------- host panel maps

struct HPanel {
    int kind;
    const double* p;
    // point on [0, 1] and its tangent / tangent norm
    void at01(double t, cplx& pt, cplx& tan, double& tn) const {
        if (kind == HBEM_PANEL_LINE) {
            double dx = p[2] - p[0], dy = p[3] - p[1];
            pt = mk(dx * t + p[0], dy * t + p[1]);
            tan = mk(dx, dy);
            tn = std::hypot(dx, dy);
        } else {
            double d = p[4] - p[3], th = t * d + p[3];
            double c = std::cos(th), s = std::sin(th);
            pt = mk(p[0] + p[2] * c, p[1] + p[2] * s);
            tan = mk(-p[2] * d * s, p[2] * d * c);
            tn = p[2] * std::fabs(d);
        }
    }
    // point on [-1, 1] (the parametrisation used by the adjacency test)
    cplx at11(double t) const {
        if (kind == HBEM_PANEL_LINE)
            return mk((t * (p[2] - p[0]) + (p[2] + p[0])) * 0.5, (t * (p[3] - p[1]) + (p[3] + p[1])) * 0.5);
        double mean = (p[3] + p[4]) / 2., diff = (p[4] - p[3]) / 2.;
        return mk(p[0] + p[2] * std::cos(t * diff + mean), p[1] + p[2] * std::sin(t * diff + mean));
    }
};

double dist(cplx a, cplx b) { return std::hypot(a.re - b.re, a.im - b.im); }

// panel-pair assembly launch with launch counting and, when enabled, CUDA-event
// timing on the launching stream
// ---- autotuner of the general-pair layout (option "autotune", default 0)
//
// The general pairs of a launch run a thread per pair or a warp per pair with ppw
// pairs per warp; the built-in rule picks by the number of pairs x jobs.  With the
// autotuner on, the first launch of each (panels, order, jobs rounded up to a power
// of two, derivative order, real k, curved) times every layout once on the launch's
// own data (CUDA events on its stream) and keeps the fastest; later launches of the
// key use it.  The choices are kept for the process and, when the environment
// variable HBEM_TUNE_CACHE names a file, read from it at the first tuned launch and
// appended to it, so later processes start tuned.  The layouts sum the same
// quadrature points in different orders: results agree to rounding (~1e-15).
constexpr int kLayoutAuto = -1;
const int kTuneLayouts[] = {0, 1, 2, 4, 8, 16};
std::atomic<int> g_autotune{0};
std::mutex g_tune_mu;
std::map<std::array<int, 6>, int> g_tune;
bool g_tune_loaded = false;

std::array<int, 6> tune_key(const DevMesh& M, int njobs, int d, bool real_k) {
    int nb = 1;
    while (nb < njobs) nb <<= 1;
    return {M.n, M.p, nb, d, real_k ? 1 : 0, M.lines ? 0 : 1};
}

void tune_load_locked() {
    g_tune_loaded = true;
    const char* f = getenv("HBEM_TUNE_CACHE");
    if (!f || !*f) return;
    FILE* fp = fopen(f, "r");
    if (!fp) return;
    std::array<int, 6> k;
    int v;
    while (fscanf(fp, "%d %d %d %d %d %d %d", &k[0], &k[1], &k[2], &k[3], &k[4], &k[5], &v) == 7) g_tune[k] = v;
    fclose(fp);
}

int tuned_layout(const DevMesh& M, const SingularTask* tasks, int ntasks, const Job* jobs, int njobs, bool real_k,
                 int d, cplx* loc, cudaStream_t st) {
    const auto key = tune_key(M, njobs, d, real_k);
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        if (!g_tune_loaded) tune_load_locked();
        auto it = g_tune.find(key);
        if (it != g_tune.end()) return it->second;
    }
    cudaEvent_t a = nullptr, b = nullptr;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return kLayoutAuto;
    int best = kLayoutAuto;
    float best_ms = 0.f;
    for (int lay : kTuneLayouts) {
        cudaEventRecord(a, st);
        if (launch_local(M, tasks, ntasks, jobs, njobs, real_k, d, loc, st, lay, 1, nullptr) != cudaSuccess) break;
        cudaEventRecord(b, st);
        if (cudaEventSynchronize(b) != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        g_launches += 1;
        if (best == kLayoutAuto || ms < best_ms) { best = lay; best_ms = ms; }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (best == kLayoutAuto) return best;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = best;
    if (const char* f = getenv("HBEM_TUNE_CACHE")) {
        if (*f) {
            if (FILE* fp = fopen(f, "a")) {
                fprintf(fp, "%d %d %d %d %d %d %d\n", key[0], key[1], key[2], key[3], key[4], key[5], best);
                fclose(fp);
            }
        }
    }
    return best;
}

// part: scratch of singular_part_bytes for the split singular launch of few jobs (or
// null: one CTA per pair and job)
cudaError_t local_assembly(const DevMesh& M, const SingularTask* tasks, int ntasks, int ncoinc, const Job* jobs,
                           int njobs, bool real_k, int d, cplx* loc, cudaStream_t st, double* part = nullptr) {
    const int layout = (g_autotune && M.n > 1) ? tuned_layout(M, tasks, ntasks, jobs, njobs, real_k, d, loc, st)
                                               : kLayoutAuto;
    cudaEvent_t e0 = nullptr;
    const bool timed = g_timing != 0;
    if (timed) timing_begin(&e0, st);
    cudaError_t e = launch_local(M, tasks, ntasks, jobs, njobs, real_k, d, loc, st, layout, 3, part);
    g_launches += (M.n > 1 ? 1 : 0) + (ntasks > 0 ? 1 : 0) + (part && singular_parts(ntasks, njobs) > 0 ? 1 : 0);
    if (timed) {
        timing_end(e0, st);
        g_asm_launches += 1;
        long long nc2 = (long long)M.nc * M.nc;
        long long nadj = ntasks - ncoinc;
        long long gen = (long long)M.n * (M.n + 1) / 2 - ntasks;
        g_asm_points += (long long)njobs * (ncoinc * nc2 + nadj * 2 * nc2 + gen * (long long)M.p * M.p);
        g_asm_split[d] += (long long)njobs * gen * M.p * M.p;
        g_asm_split[(M.sgeo ? 3 : 6) + d] += (long long)njobs * (ncoinc * nc2 + nadj * 2 * nc2);
    }
    return e;
}

}  // namespace

namespace hbem {
// error reporting for entry points defined in other translation units
int set_error(int code, const char* msg) { return fail(code, msg); }
}  // namespace hbem

// ---------------------------------------------------------------- builder

struct hbem_builder_s {
    int n = 0, p = 0, nc = 0, qtest = 2, qtrial = 2, lines = 1, device = 0;
    std::vector<int> kind;
    std::vector<double> par, xg, wg, xc, wc;
    std::vector<cplx> ends;
    std::vector<SingularTask> tasks;
    cudaStream_t st = nullptr;
    DBuf d_kind, d_par, d_xg, d_wg, d_xc, d_wc, d_gpt, d_gtan, d_gtn, d_ends, d_flags, d_tasks;
    DBuf d_loc, d_jobs, d_layers;
    DBuf d_sgeo;   // k-independent point data of the singular pairs (when within kSingularTableMax)
    DBuf d_gorder; // strictly-lower pair indices sorted by panel-midpoint distance
    int asm_layers = 0, asm_d = -1, asm_rows = 0, asm_cols = 0;

    long long npair() const { return (long long)n * (n + 1) / 2; }
    // the gather's space bits: 1 test space P0, 2 trial space P0
    int sp() const { return (qtest == HBEM_SPACE_P0 ? 1 : 0) | (qtrial == HBEM_SPACE_P0 ? 2 : 0); }
    bool p1p1() const { return qtest == HBEM_SPACE_P1 && qtrial == HBEM_SPACE_P1; }
    DevMesh view() const {
        DevMesh M;
        M.n = n; M.p = p; M.nc = nc; M.lines = lines;
        M.kind = d_kind.as<int>(); M.par = d_par.as<double>();
        M.xg = d_xg.as<double>(); M.wg = d_wg.as<double>();
        M.xc = d_xc.as<double>(); M.wc = d_wc.as<double>();
        M.gpt = d_gpt.as<cplx>(); M.gtan = d_gtan.as<cplx>(); M.gtn = d_gtn.as<double>();
        M.ends = d_ends.as<cplx>(); M.flags = d_flags.as<uint8_t>();
        M.sgeo = g_singular_table ? d_sgeo.as<double>() : nullptr;
        M.gorder = d_gorder.as<int>();
        return M;
    }
    // BuilderData::is_adjacent (galerkin_builder.cpp:189-201)
    bool adjacent(int i, int j, bool& swap) const {
        const double e = 100. * kMachEps;
        if (dist(ends[2 * i + 1], ends[2 * j]) < e) { swap = false; return true; }
        if (dist(ends[2 * i], ends[2 * j + 1]) < e) { swap = true; return true; }
        return false;
    }
    ~hbem_builder_s() {
        for (DBuf* b : {&d_kind, &d_par, &d_xg, &d_wg, &d_xc, &d_wc, &d_gpt, &d_gtan, &d_gtn, &d_ends, &d_flags,
                        &d_tasks, &d_loc, &d_jobs, &d_layers, &d_sgeo, &d_gorder})
            b->release();
        if (st) cudaStreamDestroy(st);
    }
};

// One in-flight evaluation of sigma, sigma', sigma'' at a few wavenumbers on its own
// stream (the plain search's Newton phase runs several at once): job table, pair
// blocks, T / T' / T'', results, and pinned host copies of the results.
constexpr int kLaneMaxPts = 64;
struct EvalLane {
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr, asm_done = nullptr;   // all work / the assembly part finished
    DBuf jobs, loc, T, out, status, slots;
    DBuf T2;                   // matrices from lane_launch_near's Taylor polynomials
    bool near_cur = false;     // the lane's last point's T, T', T'' are in T2 (else in T)
    double* h_out = nullptr;   // pinned, 3 x kLaneMaxPts
    int* h_status = nullptr;   // pinned, kLaneMaxPts
    int npts = 0, d = 2, mode = 0;   // mode 0: sigma (+ derivatives), 1: grid chunk, 2: bracket ends
    double k[kLaneMaxPts];
    ~EvalLane() {
        for (DBuf* x : {&jobs, &loc, &T, &out, &status, &slots, &T2}) x->release();
        if (h_out) cudaFreeHost(h_out);
        if (h_status) cudaFreeHost(h_status);
        if (done) cudaEventDestroy(done);
        if (asm_done) cudaEventDestroy(asm_done);
        if (st) cudaStreamDestroy(st);
    }
};

// Lanes are kept per host thread and device (a search runs on one thread at a time),
// so that operators created one after another reuse their streams, events and pinned
// result buffers; a lane's device buffers grow to the largest batch it has served.
struct LanePool {
    int device = -1;
    std::vector<EvalLane*> lanes;
    ~LanePool() {
        for (EvalLane* l : lanes) delete l;
    }
};
thread_local std::vector<LanePool*> t_lane_pools;
thread_local struct LanePoolsOwner {
    ~LanePoolsOwner() {
        for (LanePool* p : t_lane_pools) delete p;
    }
} t_lane_pools_owner;

LanePool& lane_pool(int device) {
    for (LanePool* p : t_lane_pools)
        if (p->device == device) return *p;
    t_lane_pools.push_back(new LanePool());
    t_lane_pools.back()->device = device;
    return *t_lane_pools.back();
}

struct hbem_solop_s {
    hbem_builder b = nullptr;
    int proj = 1;
    std::vector<double> M;    // N x N column-major
    DBuf d_M, d_id, d_sb, d_lr, d_T, d_svdA, d_svdV, d_out, d_status, d_sig;
    DBuf d_vpool, d_slots;   // FP32 V sets of the dense kernel's warm starts, slot lists
    DBuf d_uv, d_d1;         // singular vectors of sigma_min kept by sweep_sigma_warm, sigma' scratch
    int uv_count = 0;        // wavenumbers whose (u, v) d_uv holds (0: none valid)
    ~hbem_solop_s() {
        for (DBuf* x : {&d_M, &d_id, &d_sb, &d_lr, &d_T, &d_svdA, &d_svdV, &d_out, &d_status, &d_sig, &d_vpool,
                        &d_slots, &d_uv, &d_d1})
            x->release();
    }
};

// The plain search keeps up to 24 streams busy at once.  With CUDA's default of 8
// hardware work queues per device, streams share queues and a stream's launches wait
// behind another stream's (a grid chunk's event wait, a long kernel) that they do not
// depend on.  At load time, before a CUDA context exists, ask for the maximum of 32
// queues unless the process has chosen a number already.
__attribute__((constructor)) static void hbem_default_connections() {
    setenv("CUDA_DEVICE_MAX_CONNECTIONS", "32", 0);
}

extern "C" {

int hbem_version(void) { return 100; }

void hbem_stats_enable_timing(int enable) { g_timing = enable ? 1 : 0; }

void hbem_stats_reset(void) {
    g_launches = 0;
    {
        std::lock_guard<std::mutex> lk(g_stats_mu);
        resolve_pending_locked();
        g_asm_ms = 0.;
    }
    g_asm_launches = 0;
    g_asm_points = 0;
    for (auto& x : g_asm_split) x = 0;
}

void hbem_stats_read(long long* launches, double* assembly_ms, long long* assembly_launches,
                     long long* assembly_points) {
    if (launches) *launches = g_launches;
    if (assembly_ms) {
        std::lock_guard<std::mutex> lk(g_stats_mu);
        resolve_pending_locked();
        *assembly_ms = g_asm_ms;
    }
    if (assembly_launches) *assembly_launches = g_asm_launches;
    if (assembly_points) *assembly_points = g_asm_points;
}

void hbem_stats_read_points(long long* split9) {
    if (split9)
        for (int i = 0; i < 9; ++i) split9[i] = g_asm_split[i];
}

const char* hbem_status_string(int s) {
    switch (s) {
        case HBEM_OK: return "ok";
        case HBEM_ERR_INVALID: return "invalid argument";
        case HBEM_ERR_CUDA: return "CUDA error";
        case HBEM_ERR_NOMEM: return "out of device memory";
        case HBEM_ERR_NOCONV: return "iteration limit reached";
        case HBEM_ERR_SINGULAR: return "singular pivot";
        case HBEM_ERR_NONFINITE: return "non-finite value";
        case HBEM_ERR_UNSUPPORTED: return "unsupported";
        default: return "unknown status";
    }
}

const char* hbem_last_error(void) { return g_err.c_str(); }

int hbem_set_device(int device) {
    HB_CK(cudaSetDevice(device));
    g_device = device;
    return HBEM_OK;
}

int hbem_set_option(const char* name, int value) {
    if (!name) return fail(HBEM_ERR_INVALID, "set_option: no name");
    const std::string k(name);
    if (k == "lu_cluster_panels") {
        lu_set_cluster_panels(value);
        return HBEM_OK;
    }
    if (k == "lu_tensor_cores") {
        lu_set_tensor_cores(value);
        return HBEM_OK;
    }
    if (k == "svd_fast") {
        g_svd_fast = value ? 1 : 0;
        return HBEM_OK;
    }
    if (k == "svd_pair_max") {
        if (value < 0) return fail(HBEM_ERR_INVALID, "set_option: svd_pair_max must be >= 0");
        svd_set_pair_max(value);
        return HBEM_OK;
    }
    if (k == "autotune") {
        g_autotune = value ? 1 : 0;
        return HBEM_OK;
    }
    if (k == "svd_fast_force_redo") {
        g_svd_force_redo = value ? 1 : 0;
        return HBEM_OK;
    }
    if (k == "mlp_tensor_cores") {
        mlp_set_tensor_cores(value);
        return HBEM_OK;
    }
    if (k == "singular_table") {
        g_singular_table = value ? 1 : 0;
        return HBEM_OK;
    }
    if (k == "plain_warm_start") {
        g_plain_warm_start = value ? 1 : 0;
        return HBEM_OK;
    }
    if (k == "singular_split") {
        g_singular_split = value ? 1 : 0;
        return HBEM_OK;
    }
    if (k == "plain_speculate") {
        g_plain_speculate = value ? 1 : 0;
        return HBEM_OK;
    }
    if (k == "plain_async") {
        g_plain_async = value ? 1 : 0;
        return HBEM_OK;
    }
    if (k == "plain_spec_async") {
        if (value < 0) return fail(HBEM_ERR_INVALID, "set_option: plain_spec_async must be >= 0");
        g_plain_spec_async = value;
        return HBEM_OK;
    }
    if (k == "plain_spec_deep") {
        if (value < 0) return fail(HBEM_ERR_INVALID, "set_option: plain_spec_deep must be >= 0");
        g_plain_spec_deep = value;
        return HBEM_OK;
    }
    if (k == "arnoldi_maxit") {
        if (value < 1) return fail(HBEM_ERR_INVALID, "set_option: arnoldi_maxit must be >= 1");
        g_arnoldi_maxit = value;
        return HBEM_OK;
    }
    return fail(HBEM_ERR_INVALID, "set_option: unknown option " + k);
}

int hbem_get_option(const char* name, int* value) {
    if (!name || !value) return fail(HBEM_ERR_INVALID, "get_option: bad argument");
    const std::string k(name);
    if (k == "lu_cluster_panels") *value = lu_get_cluster_panels();
    else if (k == "lu_tensor_cores") *value = lu_get_tensor_cores();
    else if (k == "svd_fast") *value = g_svd_fast.load();
    else if (k == "svd_pair_max") *value = svd_get_pair_max();
    else if (k == "svd_fast_force_redo") *value = g_svd_force_redo.load();
    else if (k == "autotune") *value = g_autotune.load();
    else if (k == "mlp_tensor_cores") *value = mlp_get_tensor_cores();
    else if (k == "singular_table") *value = g_singular_table;
    else if (k == "plain_warm_start") *value = g_plain_warm_start;
    else if (k == "singular_split") *value = g_singular_split;
    else if (k == "plain_speculate") *value = g_plain_speculate;
    else if (k == "plain_async") *value = g_plain_async;
    else if (k == "plain_spec_async") *value = g_plain_spec_async;
    else if (k == "plain_spec_deep") *value = g_plain_spec_deep;
    else if (k == "arnoldi_maxit") *value = g_arnoldi_maxit;
    else return fail(HBEM_ERR_INVALID, "get_option: unknown option " + k);
    return HBEM_OK;
}

int hbem_hankel01(int n, const double* z_host, int complex_arg, double* h0_host, double* h1_host) {
    if (n < 1 || !z_host || !h0_host || !h1_host) return fail(HBEM_ERR_INVALID, "hankel01: bad argument");
    HB_CK(cudaSetDevice(g_device));
    static thread_local DBuf z, a, b;
    const size_t bytes = (size_t)n * sizeof(cplx);
    HB_CK(z.ensure(bytes));
    HB_CK(a.ensure(bytes));
    HB_CK(b.ensure(bytes));
    std::vector<cplx> zz(n);
    for (int i = 0; i < n; ++i) zz[i] = complex_arg ? mk(z_host[2 * i], z_host[2 * i + 1]) : mk(z_host[i], 0.);
    HB_CK(cudaMemcpy(z.p, zz.data(), bytes, cudaMemcpyHostToDevice));
    HB_CK(launch_hankel01(n, z.as<cplx>(), complex_arg, a.as<cplx>(), b.as<cplx>(), 0));
    HB_CK(cudaMemcpy(h0_host, a.p, bytes, cudaMemcpyDeviceToHost));
    HB_CK(cudaMemcpy(h1_host, b.p, bytes, cudaMemcpyDeviceToHost));
    return HBEM_OK;
}

int hbem_builder_create(int npanels, const int* kinds, const double* params, int order, int q_test, int q_trial,
                        hbem_builder* out) {
    if (!out || !kinds || !params || npanels < 3 || order < 2 || order > 32)
        return fail(HBEM_ERR_INVALID, "builder: need >= 3 panels and 2 <= order <= 32");
    if ((q_test != HBEM_SPACE_P0 && q_test != HBEM_SPACE_P1) || (q_trial != HBEM_SPACE_P0 && q_trial != HBEM_SPACE_P1))
        return fail(HBEM_ERR_INVALID, "builder: spaces are P0 (1) or P1 (2)");
    for (int i = 0; i < npanels; ++i)
        if (kinds[i] != HBEM_PANEL_LINE && kinds[i] != HBEM_PANEL_ARC) return fail(HBEM_ERR_INVALID, "builder: bad panel kind");
    HB_CK(cudaSetDevice(g_device));
    hbem_builder b = new hbem_builder_s();
    b->device = g_device;
    b->n = npanels; b->p = order; b->nc = order * (order + 1) / 2 - 1;
    b->qtest = q_test; b->qtrial = q_trial;
    b->kind.assign(kinds, kinds + npanels);
    b->par.assign(params, params + 5 * (size_t)npanels);
    b->lines = 1;
    for (int k : b->kind) if (k != HBEM_PANEL_LINE) b->lines = 0;
    b->xg.resize(order); b->wg.resize(order);
    gauss_legendre(0., 1., order, b->xg.data(), b->wg.data());
    b->xc.resize(b->nc); b->wc.resize(b->nc);
    graded_composite(order, b->xc.data(), b->wc.data());
    // geometry at the general nodes and panel end points
    const int n = npanels, p = order;
    std::vector<cplx> gpt((size_t)n * p), gtan((size_t)n * p);
    std::vector<double> gtn((size_t)n * p);
    b->ends.resize(2 * (size_t)n);
    for (int i = 0; i < n; ++i) {
        HPanel P{b->kind[i], &b->par[5 * (size_t)i]};
        for (int a = 0; a < p; ++a) P.at01(b->xg[a], gpt[(size_t)i * p + a], gtan[(size_t)i * p + a], gtn[(size_t)i * p + a]);
        b->ends[2 * i] = P.at11(-1.);
        b->ends[2 * i + 1] = P.at11(1.);
    }
    // pair classification (coincident / adjacent) -> singular task list, flag bit 7
    std::vector<uint8_t> flags((size_t)b->npair(), 0);
    for (int i = 0; i < n; ++i) {
        b->tasks.push_back(SingularTask{i, i, PK_COINC, 0});
        flags[tri_index(i, i)] = 0x80;
        for (int j = 0; j < i; ++j) {
            bool sw = false;
            if (b->adjacent(i, j, sw)) {
                b->tasks.push_back(SingularTask{i, j, PK_ADJ, sw ? 1 : 0});
                flags[tri_index(i, j)] = 0x80;
            }
        }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = upload(b->d_kind, b->kind, b->st);
    if (e == cudaSuccess) e = upload(b->d_par, b->par, b->st);
    if (e == cudaSuccess) e = upload(b->d_xg, b->xg, b->st);
    if (e == cudaSuccess) e = upload(b->d_wg, b->wg, b->st);
    if (e == cudaSuccess) e = upload(b->d_xc, b->xc, b->st);
    if (e == cudaSuccess) e = upload(b->d_wc, b->wc, b->st);
    if (e == cudaSuccess) e = upload(b->d_gpt, gpt, b->st);
    if (e == cudaSuccess) e = upload(b->d_gtan, gtan, b->st);
    if (e == cudaSuccess) e = upload(b->d_gtn, gtn, b->st);
    if (e == cudaSuccess) e = upload(b->d_ends, b->ends, b->st);
    if (e == cudaSuccess) e = upload(b->d_flags, flags, b->st);
    if (e == cudaSuccess) e = upload(b->d_tasks, b->tasks, b->st);
    if (e == cudaSuccess) e = launch_flags(b->view(), b->d_tasks.as<SingularTask>(), (int)b->tasks.size(),
                                           b->d_flags.as<uint8_t>(), b->st);
    // general pairs in order of the distance between their panels' middle Gauss points
    // (ties by index): the thread-per-pair kernel's warps then see similar distances
    if (e == cudaSuccess && n > 1 && (long long)n * (n - 1) / 2 < (1LL << 31)) {
        const long long nlow = (long long)n * (n - 1) / 2;
        std::vector<float> key((size_t)nlow);
        std::vector<int> ord((size_t)nlow);
        for (long long i = 1, q = 0; i < n; ++i)
            for (long long j = 0; j < i; ++j, ++q) {
                const cplx a = gpt[(size_t)i * p + p / 2], c = gpt[(size_t)j * p + p / 2];
                key[(size_t)q] = (float)std::hypot(a.re - c.re, a.im - c.im);
                ord[(size_t)q] = (int)q;
            }
        std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return key[(size_t)x] < key[(size_t)y]; });
        e = upload(b->d_gorder, ord, b->st);
    }
    const size_t geo_bytes = singular_geo_bytes(b->nc, (int)b->tasks.size());
    if (e == cudaSuccess && geo_bytes > 0 && geo_bytes <= kSingularTableMax) {
        e = b->d_sgeo.ensure(geo_bytes);
        if (e == cudaSuccess) {
            DevMesh M = b->view();
            M.sgeo = nullptr;
            e = launch_singular_geo(M, b->d_tasks.as<SingularTask>(), (int)b->tasks.size(), b->d_sgeo.as<double>(),
                                    b->st);
        }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) {
        std::string msg = cudaGetErrorString(e);
        delete b;
        return fail(e == cudaErrorMemoryAllocation ? HBEM_ERR_NOMEM : HBEM_ERR_CUDA, "builder: " + msg);
    }
    *out = b;
    return HBEM_OK;
}

int hbem_builder_destroy(hbem_builder b) {
    delete b;
    return HBEM_OK;
}

int hbem_builder_info(hbem_builder b, int* npanels, int* dim_test, int* dim_trial, int* order, int* lines) {
    if (!b) return fail(HBEM_ERR_INVALID, "null builder");
    if (npanels) *npanels = b->n;
    if (dim_test) *dim_test = b->n;
    if (dim_trial) *dim_trial = b->n;
    if (order) *order = b->p;
    if (lines) *lines = b->lines;
    return HBEM_OK;
}

int hbem_builder_is_adjacent(hbem_builder b, int i, int j, int* adjacent, int* swap) {
    if (!b || i < 0 || j < 0 || i >= b->n || j >= b->n) return fail(HBEM_ERR_INVALID, "is_adjacent: bad index");
    bool sw = false;
    bool a = b->adjacent(i, j, sw);
    if (adjacent) *adjacent = a;
    if (swap) *swap = sw;
    return HBEM_OK;
}

static int check_kc(double k_im, double c) {
    if (!(c >= 1.)) return fail(HBEM_ERR_INVALID, "Refraction index must not be smaller than 1");
    if (k_im < 0.) return fail(HBEM_ERR_INVALID, "Wavenumber does not meet conditions for uniqueness of the solution (Im(k) >= 0)");
    return HBEM_OK;
}

int hbem_assemble_dense(hbem_builder b, double k_re, double k_im, double c, unsigned layers, unsigned d) {
    return hbem_assemble_dense_sub(b, k_re, k_im, c, layers, d, 0, 0, 0, 0);
}

int hbem_assemble_dense_sub(hbem_builder b, double k_re, double k_im, double c, unsigned layers, unsigned d,
                            unsigned row, unsigned col, unsigned rows, unsigned cols) {
    if (!b) return fail(HBEM_ERR_INVALID, "null builder");
    if (rows == 0) rows = (unsigned)b->n;
    if (cols == 0) cols = (unsigned)b->n;
    if ((size_t)row + rows > (size_t)b->n || (size_t)col + cols > (size_t)b->n)
        return fail(HBEM_ERR_INVALID, "sub-matrix outside the panel range");
    if (int r = check_kc(k_im, c)) return r;
    if (d > 2) return fail(HBEM_ERR_INVALID, "Invalid order of derivative");
    if (layers == 0 || layers > 7) return fail(HBEM_ERR_INVALID, "bad layer mask");
    HB_CK(cudaSetDevice(b->device));
    const long long np = b->npair();
    const size_t loc_bytes = (size_t)np * (d + 1) * kLocPerD * sizeof(cplx);
    HB_CK(b->d_loc.ensure(loc_bytes));
    std::vector<Job> jobs{Job{k_re, k_im, c}};
    HB_CK(upload(b->d_jobs, jobs, b->st));
    int nl = ((layers & 1) != 0) + ((layers & 2) != 0) + ((layers & 4) != 0);
    HB_CK(b->d_layers.ensure((size_t)nl * (d + 1) * rows * cols * sizeof(cplx)));
    bool real_k = (k_im == 0. && k_re > 0.);
    HB_CK(local_assembly(b->view(), b->d_tasks.as<SingularTask>(), (int)b->tasks.size(), b->n, b->d_jobs.as<Job>(), 1,
                         real_k, (int)d, b->d_loc.as<cplx>(), b->st));
    if (rows == (unsigned)b->n && cols == (unsigned)b->n)
        HB_CK(launch_gather_layers(b->n, (int)d, (int)layers, b->d_loc.as<cplx>(), 0, b->sp(), b->d_layers.as<cplx>(),
                                   b->st));
    else
        HB_CK(launch_gather_layers_sub(b->n, (int)d, (int)layers, b->d_loc.as<cplx>(), 0, (int)row, (int)rows,
                                       (int)col, (int)cols, b->sp(), b->d_layers.as<cplx>(), b->st));
    g_launches += 1;
    HB_CK(cudaStreamSynchronize(b->st));
    b->asm_layers = (int)layers;
    b->asm_d = (int)d;
    b->asm_rows = (int)rows;
    b->asm_cols = (int)cols;
    return HBEM_OK;
}

static int layer_slot(hbem_builder b, unsigned layer, unsigned d, size_t* off) {
    if (!b) return fail(HBEM_ERR_INVALID, "null builder");
    if (d > 2 || (int)d > b->asm_d) return fail(HBEM_ERR_INVALID, "Invalid order of derivative");
    if (layer != HBEM_LAYER_DOUBLE && layer != HBEM_LAYER_SINGLE && layer != HBEM_LAYER_HYPERSINGULAR)
        return fail(HBEM_ERR_INVALID, "bad layer");
    if (!(b->asm_layers & (int)layer)) return fail(HBEM_ERR_INVALID, "Requested layer is not computed, so cannot be retrieved");
    // slots in the order K, W, V
    int slot = 0;
    const int order[3] = {HBEM_LAYER_DOUBLE, HBEM_LAYER_HYPERSINGULAR, HBEM_LAYER_SINGLE};
    for (int L : order) {
        if ((unsigned)L == layer) break;
        if (b->asm_layers & L) ++slot;
    }
    *off = ((size_t)slot * (b->asm_d + 1) + d) * b->asm_rows * b->asm_cols;
    return HBEM_OK;
}

int hbem_get_layer(hbem_builder b, unsigned layer, unsigned d, double* host_out) {
    size_t off;
    if (int r = layer_slot(b, layer, d, &off)) return r;
    if (!host_out) return fail(HBEM_ERR_INVALID, "null output");
    HB_CK(cudaMemcpy(host_out, b->d_layers.as<cplx>() + off, (size_t)b->asm_rows * b->asm_cols * sizeof(cplx),
                     cudaMemcpyDeviceToHost));
    return HBEM_OK;
}

int hbem_get_layer_device(hbem_builder b, unsigned layer, unsigned d, const void** dev_ptr) {
    size_t off;
    if (int r = layer_slot(b, layer, d, &off)) return r;
    if (!dev_ptr) return fail(HBEM_ERR_INVALID, "null output");
    *dev_ptr = b->d_layers.as<cplx>() + off;
    return HBEM_OK;
}

// ---------------------------------------------------------------- solutions operator

int hbem_solop_create(hbem_builder b, int proj, hbem_solop* out) {
    if (!b || !out) return fail(HBEM_ERR_INVALID, "null argument");
    HB_CK(cudaSetDevice(b->device));
    const int N = b->n;
    if (proj && b->qtest != b->qtrial)
        return fail(HBEM_ERR_UNSUPPORTED,
                    "solutions operator: the projection needs test space = trial space (the mass matrix of P0 x P1 "
                    "is not symmetric)");
    hbem_solop s = new hbem_solop_s();
    s->b = b;
    s->proj = proj ? 1 : 0;
    // mass matrix (mass_matrix.cpp:6-47): 2*max(q) Gauss points for line meshes, the
    // builder's order otherwise (gen_sol_op.cpp:29-32)
    const int mo = b->lines ? 2 * std::max(b->qtest, b->qtrial) : b->p;
    std::vector<double> x(mo), w(mo);
    gauss_legendre(0., 1., mo, x.data(), w.data());
    // local functions (continuous_space.hpp:38-47, discontinuous_space.hpp:38-44): P1
    // t (dof i + 1) and 1 - t (dof i) on panel i; P0 the constant 1 (dof i)
    auto shape = [](int q, int l, double t) { return q == HBEM_SPACE_P0 ? 1. : (l == 0 ? t : 1. - t); };
    auto dof = [N](int q, int l, int i) { return q == HBEM_SPACE_P0 ? i : (l == 0 ? (i + 1) % N : i); };
    s->M.assign((size_t)N * N, 0.);
    for (int i = 0; i < N; ++i) {
        HPanel P{b->kind[i], &b->par[5 * (size_t)i]};
        for (int ii = 0; ii < b->qtest; ++ii)
            for (int jj = 0; jj < b->qtrial; ++jj) {
                int II = dof(b->qtest, ii, i), JJ = dof(b->qtrial, jj, i);
                double sum = 0.;
                for (int k = 0; k < mo; ++k) {
                    cplx pt, tan;
                    double tn;
                    P.at01(x[k], pt, tan, tn);
                    double F = shape(b->qtrial, jj, x[k]) * tn, G = shape(b->qtest, ii, x[k]);
                    sum = sum + w[k] * F * G;
                }
                s->M[II + (size_t)JJ * N] += sum;
            }
    }
    cudaError_t e = upload(s->d_M, s->M, b->st);
    if (e == cudaSuccess && s->proj) {
        // Cholesky of the cyclic tridiagonal M: bidiagonal + dense last row
        std::vector<double> id(N), sb(N, 0.), lr(N, 0.);
        auto Mv = [&](int r, int c) { return s->M[r + (size_t)c * N]; };
        double last_prev = 0., sub_prev = 0.;
        bool ok = true;
        for (int i = 0; i < N - 1; ++i) {
            double dd = Mv(i, i) - (i > 0 ? sub_prev * sub_prev : 0.);
            if (!(dd > 0.)) { ok = false; break; }
            double di = std::sqrt(dd);
            id[i] = 1. / di;
            double sub = (i + 1 < N - 1) ? Mv(i + 1, i) / di : 0.;
            double l = (Mv(N - 1, i) - (i > 0 ? last_prev * sub_prev : 0.)) / di;
            lr[i] = l;
            if (i + 1 < N - 1) sb[i] = sub;
            else sb[i] = l;   // L[N-1][N-2] is part of the last row
            last_prev = l;
            sub_prev = sub;
        }
        if (ok) {
            double dd = Mv(N - 1, N - 1);
            for (int i = 0; i < N - 1; ++i) dd -= lr[i] * lr[i];
            if (!(dd > 0.)) ok = false;
            else id[N - 1] = 1. / std::sqrt(dd);
        }
        if (!ok) {
            delete s;
            return fail(HBEM_ERR_SINGULAR, "mass matrix is not positive definite");
        }
        e = upload(s->d_id, id, b->st);
        if (e == cudaSuccess) e = upload(s->d_sb, sb, b->st);
        if (e == cudaSuccess) e = upload(s->d_lr, lr, b->st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) {
        delete s;
        return fail(HBEM_ERR_CUDA, std::string("solop: ") + cudaGetErrorString(e));
    }
    *out = s;
    return HBEM_OK;
}

int hbem_solop_destroy(hbem_solop s) {
    delete s;
    return HBEM_OK;
}

int hbem_mass_matrix(hbem_solop s, double* host_out) {
    if (!s || !host_out) return fail(HBEM_ERR_INVALID, "null argument");
    std::memcpy(host_out, s->M.data(), s->M.size() * sizeof(double));
    return HBEM_OK;
}

// T(k) (+ derivatives) for nk wavenumbers into T_dev [nk][d+1][2N][2N]; k_host may be complex
// (interleaved) when kim_host != NULL.
static int gen_T_batch_ws(hbem_solop s, const double* k_host, const double* kim_host, int nk, double c_o, double c_i,
                          unsigned d, cplx* T_dev, DBuf& d_jobs, DBuf& d_loc, cudaStream_t st);

static int gen_T_batch(hbem_solop s, const double* k_host, const double* kim_host, int nk, double c_o, double c_i,
                       unsigned d, cplx* T_dev) {
    return gen_T_batch_ws(s, k_host, kim_host, nk, c_o, c_i, d, T_dev, s->b->d_jobs, s->b->d_loc, s->b->st);
}

// T(k) batch with the job table and pair-block scratch given, on stream st
static int gen_T_batch_ws(hbem_solop s, const double* k_host, const double* kim_host, int nk, double c_o, double c_i,
                          unsigned d, cplx* T_dev, DBuf& d_jobs, DBuf& d_loc, cudaStream_t st) {
    hbem_builder b = s->b;
    const int N = b->n;
    const long long np = b->npair();
    const size_t per_job = (size_t)np * (d + 1) * kLocPerD * sizeof(cplx);
    // bound the pair-local scratch to 4 GiB per launch group
    int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)nk, ((size_t)4 << 30) / (2 * per_job)));
    const size_t mat = 4ULL * N * N;
    for (int k0 = 0; k0 < nk; k0 += chunk) {
        int kn = std::min(chunk, nk - k0);
        std::vector<Job> jobs;
        bool real_k = true;
        for (int q = 0; q < kn; ++q) {
            double kr = k_host[k0 + q], ki = kim_host ? kim_host[k0 + q] : 0.;
            if (int r = check_kc(ki, c_i)) return r;
            if (int r = check_kc(ki, c_o)) return r;
            if (!(ki == 0. && kr > 0.)) real_k = false;
            jobs.push_back(Job{kr, ki, c_i});
            jobs.push_back(Job{kr, ki, c_o});
        }
        HB_CK(upload(d_jobs, jobs, st));
        // the pair blocks, then the partial sums of a split singular launch
        const size_t part_bytes =
            (g_singular_split && !t_split_hold) ? singular_part_bytes((int)b->tasks.size(), 2 * kn, (int)d, !b->lines)
                                                : 0;
        HB_CK(d_loc.ensure(per_job * 2 * kn + part_bytes));
        double* part = part_bytes ? reinterpret_cast<double*>(d_loc.as<char>() + per_job * 2 * kn) : nullptr;
        HB_CK(local_assembly(b->view(), b->d_tasks.as<SingularTask>(), (int)b->tasks.size(), b->n, d_jobs.as<Job>(),
                             2 * kn, real_k, (int)d, d_loc.as<cplx>(), st, part));
        cplx* Tk = T_dev + (size_t)k0 * (d + 1) * mat;
        HB_CK(launch_gather_T(N, (int)d, d_loc.as<cplx>(), s->d_M.as<double>(), kn, b->sp(), Tk, st));
        g_launches += 1;
        if (s->proj) {
            HB_CK(launch_projection(N, s->d_id.as<double>(), s->d_sb.as<double>(), s->d_lr.as<double>(), Tk,
                                    kn * (int)(d + 1), st));
            g_launches += 2;
        }
    }
    return HBEM_OK;
}

int hbem_gen_sol_op(hbem_solop s, double k_re, double k_im, double c_o, double c_i, unsigned d, double* T_host) {
    if (!s || !T_host) return fail(HBEM_ERR_INVALID, "null argument");
    if (d > 2) return fail(HBEM_ERR_INVALID, "Invalid order of derivative");
    hbem_builder b = s->b;
    HB_CK(cudaSetDevice(b->device));
    const size_t mat = 4ULL * b->n * b->n;
    HB_CK(s->d_T.ensure((d + 1) * mat * sizeof(cplx)));
    if (int r = gen_T_batch(s, &k_re, &k_im, 1, c_o, c_i, d, s->d_T.as<cplx>())) return r;
    HB_CK(cudaMemcpyAsync(T_host, s->d_T.p, (d + 1) * mat * sizeof(cplx), cudaMemcpyDeviceToHost, b->st));
    HB_CK(cudaStreamSynchronize(b->st));
    return HBEM_OK;
}

int hbem_gen_sol_op_batch_device(hbem_solop s, const double* k_host, int nk, double c_o, double c_i, unsigned d,
                                 void* T_dev) {
    if (!s || !k_host || !T_dev || nk < 1) return fail(HBEM_ERR_INVALID, "bad argument");
    if (d > 2) return fail(HBEM_ERR_INVALID, "Invalid order of derivative");
    HB_CK(cudaSetDevice(s->b->device));
    if (int r = gen_T_batch(s, k_host, nullptr, nk, c_o, c_i, d, static_cast<cplx*>(T_dev))) return r;
    HB_CK(cudaStreamSynchronize(s->b->st));
    return HBEM_OK;
}

// Several operators (scatterers of uneven panel counts) at their own wavenumbers: the
// pair blocks of every (scatterer, k, medium) job in one general-pair and one
// singular-pair launch per group of meshes of one panel kind, then each operator's
// gather and projection, all on the first operator's stream.
int hbem_gen_sol_op_multi_device(const hbem_solop* ops, int nops, const int* counts, const double* k_host,
                                 const double* c_i_host, double c_o, unsigned d, void* const* T_dev) {
    if (!ops || nops < 1 || !counts || !k_host || !c_i_host || !T_dev || d > 2)
        return fail(HBEM_ERR_INVALID, "gen_sol_op_multi: bad argument");
    for (int i = 0; i < nops; ++i) {
        if (!ops[i] || counts[i] < 0 || (counts[i] > 0 && !T_dev[i]))
            return fail(HBEM_ERR_INVALID, "gen_sol_op_multi: bad argument");
        if (ops[i]->b->device != ops[0]->b->device)
            return fail(HBEM_ERR_INVALID, "gen_sol_op_multi: operators on different devices");
        if (int r = check_kc(0., c_i_host[i])) return r;
    }
    if (int r = check_kc(0., c_o)) return r;
    std::vector<size_t> koff(nops + 1, 0);
    for (int i = 0; i < nops; ++i) {
        koff[i + 1] = koff[i] + (size_t)counts[i];
        for (int q = 0; q < counts[i]; ++q)
            if (!(k_host[koff[i] + q] > 0.))
                return fail(HBEM_ERR_INVALID, "gen_sol_op_multi: wavenumbers must be real and positive");
    }
    hbem_builder b0 = ops[0]->b;
    HB_CK(cudaSetDevice(b0->device));
    cudaStream_t st = b0->st;
    // the other operators' streams may still hold work on their buffers
    for (int i = 1; i < nops; ++i) HB_CK(cudaStreamSynchronize(ops[i]->b->st));
    // job table and pair-block scratch: the first operator's builder's buffers
    static thread_local DBuf d_meshes, d_start;
    DBuf& d_jobs = b0->d_jobs;
    DBuf& d_loc = b0->d_loc;
    std::vector<MultiMesh> meshes(nops);
    int max_nc = 0;
    for (int i = 0; i < nops; ++i) {
        meshes[i] = MultiMesh{ops[i]->b->view(), ops[i]->b->d_tasks.as<SingularTask>(), (int)ops[i]->b->tasks.size()};
        max_nc = std::max(max_nc, ops[i]->b->nc);
    }
    HB_CK(upload(d_meshes, meshes, st));
    const size_t per_pair = (size_t)(d + 1) * kLocPerD;   // complex entries per pair and job
    const size_t budget = ((size_t)4 << 30) / sizeof(cplx);
    size_t kmax = 0;
    for (int i = 0; i < nops; ++i) kmax = std::max(kmax, (size_t)counts[i]);
    for (int curved = 0; curved < 2; ++curved) {
        // wavenumber chunks: every operator of the group advances by `chunk` wavenumbers
        // per launch pair, within the 4 GiB scratch bound
        size_t per_k = 0;
        for (int i = 0; i < nops; ++i)
            if ((ops[i]->b->lines == 0) == (curved == 1)) per_k += 2 * (size_t)ops[i]->b->npair() * per_pair;
        if (per_k == 0) continue;
        const size_t chunk = std::max<size_t>(1, budget / per_k);
        for (size_t q0 = 0; q0 < kmax; q0 += chunk) {
            std::vector<MultiJob> jobs;
            std::vector<long long> gstart{0}, sstart{0};
            std::vector<size_t> first(nops, 0), nk(nops, 0);
            long long off = 0;
            for (int i = 0; i < nops; ++i) {
                hbem_builder b = ops[i]->b;
                if ((b->lines == 0) != (curved == 1) || (size_t)counts[i] <= q0) continue;
                nk[i] = std::min(chunk, (size_t)counts[i] - q0);
                first[i] = jobs.size();
                const long long nlow = (long long)b->n * (b->n - 1) / 2;
                for (size_t q = 0; q < nk[i]; ++q) {
                    const double k = k_host[koff[i] + q0 + q];
                    for (double c : {c_i_host[i], c_o}) {
                        jobs.push_back(MultiJob{Job{k, 0., c}, i, off});
                        off += (long long)(b->npair() * per_pair);
                        gstart.push_back(gstart.back() + (nlow + 127) / 128);
                        sstart.push_back(sstart.back() + (long long)b->tasks.size());
                    }
                }
            }
            if (jobs.empty()) continue;
            const int njobs = (int)jobs.size();
            std::vector<long long> starts(gstart);
            starts.insert(starts.end(), sstart.begin(), sstart.end());
            HB_CK(upload(d_jobs, jobs, st));
            HB_CK(upload(d_start, starts, st));
            HB_CK(d_loc.ensure((size_t)off * sizeof(cplx)));
            cudaEvent_t e0 = nullptr;
            const bool timed = g_timing != 0;
            if (timed) timing_begin(&e0, st);
            HB_CK(launch_local_multi(d_meshes.as<MultiMesh>(), d_jobs.as<MultiJob>(), njobs, d_start.as<long long>(),
                                     gstart.back(), d_start.as<long long>() + gstart.size(), sstart.back(), max_nc,
                                     curved == 1, true, (int)d, d_loc.as<cplx>(), st));
            g_launches += (gstart.back() > 0 ? 1 : 0) + (sstart.back() > 0 ? 1 : 0);
            if (timed) {
                timing_end(e0, st);
                g_asm_launches += 1;
                for (int i = 0; i < nops; ++i) {
                    if (!nk[i]) continue;
                    const hbem_builder b = ops[i]->b;
                    const long long nc2 = (long long)b->nc * b->nc, ntasks = (long long)b->tasks.size();
                    const long long ncoinc = b->n, nadj = ntasks - ncoinc;
                    const long long gen = b->npair() - ntasks;
                    const long long nj = 2LL * (long long)nk[i];
                    g_asm_points += nj * (ncoinc * nc2 + nadj * 2 * nc2 + gen * (long long)b->p * b->p);
                    g_asm_split[d] += nj * gen * b->p * b->p;
                    g_asm_split[(b->d_sgeo.p && g_singular_table ? 3 : 6) + d] += nj * (ncoinc * nc2 + nadj * 2 * nc2);
                }
            }
            for (int i = 0; i < nops; ++i) {
                if (!nk[i]) continue;
                hbem_solop s = ops[i];
                const int N = s->b->n;
                const size_t mat = 4ULL * N * N;
                cplx* Tk = static_cast<cplx*>(T_dev[i]) + q0 * (d + 1) * mat;
                HB_CK(launch_gather_T(N, (int)d, d_loc.as<cplx>() + jobs[first[i]].loc, s->d_M.as<double>(),
                                      (int)nk[i], s->b->sp(), Tk, st));
                g_launches += 1;
                if (s->proj) {
                    HB_CK(launch_projection(N, s->d_id.as<double>(), s->d_sb.as<double>(), s->d_lr.as<double>(), Tk,
                                            (int)nk[i] * (int)(d + 1), st));
                    g_launches += 2;
                }
            }
        }
    }
    HB_CK(cudaStreamSynchronize(st));
    return HBEM_OK;
}

// ---------------------------------------------------------------- singular values

static int sv_batch(cudaStream_t st, int n, int nmat, unsigned d, const cplx* T, long long mat_stride,
                    long long der_stride, DBuf& A, DBuf& V, DBuf& out, DBuf& status, DBuf* sig, double* out_host,
                    double* sig_all_host, cplxf* vpool = nullptr, const int* warm_slot = nullptr,
                    const int* out_slot = nullptr, cplx* uv = nullptr, int* fast_ok = nullptr) {
    if (fast_ok) *fast_ok = 0;
    const size_t nn = (size_t)n * n;
    HB_CK(V.ensure((size_t)nmat * nn * sizeof(cplx)));
    HB_CK(A.ensure(n > 100 ? (size_t)nmat * nn * sizeof(cplx) : sizeof(cplx)));
    HB_CK(out.ensure((size_t)nmat * 3 * sizeof(double)));
    HB_CK(status.ensure((size_t)nmat * sizeof(int)));
    double* dsig = nullptr;
    if (sig_all_host) {
        HB_CK(sig->ensure((size_t)nmat * n * sizeof(double)));
        dsig = sig->as<double>();
    }
    std::vector<int> stat(nmat);
    if (!sig_all_host && svd_fast_on() && svd_fast_smem_bytes(n) <= 220 * 1024) {
        // FP32 Jacobi + FP64 refinement; matrices it cannot finish (singular T, a
        // far-field series that does not converge) are redone by the polished kernel
        HB_CK(launch_svd_fast(n, nmat, (int)d, T, mat_stride, der_stride, out.as<double>(), status.as<int>(), st,
                              vpool, warm_slot, out_slot, uv));
        g_launches += 1;
        HB_CK(cudaMemcpyAsync(stat.data(), status.p, (size_t)nmat * sizeof(int), cudaMemcpyDeviceToHost, st));
        HB_CK(cudaStreamSynchronize(st));
        bool redo = g_svd_force_redo.load(std::memory_order_relaxed) != 0;
        for (int v : stat) redo |= v != 0;
        if (!redo) {
            HB_CK(cudaMemcpyAsync(out_host, out.p, (size_t)nmat * 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
            HB_CK(cudaStreamSynchronize(st));
            if (fast_ok) *fast_ok = 1;
            return HBEM_OK;
        }
    }
    HB_CK(launch_svd_mixed(n, nmat, (int)d, 0, T, mat_stride, der_stride, A.as<cplx>(), V.as<cplx>(),
                           out.as<double>(), dsig, status.as<int>(), st));
    g_launches += 1;
    HB_CK(cudaMemcpyAsync(out_host, out.p, (size_t)nmat * 3 * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (sig_all_host)
        HB_CK(cudaMemcpyAsync(sig_all_host, dsig, (size_t)nmat * n * sizeof(double), cudaMemcpyDeviceToHost, st));
    HB_CK(cudaMemcpyAsync(stat.data(), status.p, (size_t)nmat * sizeof(int), cudaMemcpyDeviceToHost, st));
    HB_CK(cudaStreamSynchronize(st));
    for (int v : stat)
        if (v) return fail(HBEM_ERR_NOCONV, "Jacobi SVD: sweep limit reached");
    return HBEM_OK;
}

int hbem_sv_dense_batch_device(int n, int nmat, unsigned d, const void* T_dev, long long mat_stride,
                               long long der_stride, double* out_host, double* sig_all_host) {
    if (n < 2 || nmat < 1 || !T_dev || !out_host || d > 2) return fail(HBEM_ERR_INVALID, "bad argument");
    HB_CK(cudaSetDevice(g_device));
    static thread_local DBuf A, V, out, status, sig;
    return sv_batch(0, n, nmat, d, static_cast<const cplx*>(T_dev), mat_stride, der_stride, A, V, out, status, &sig,
                    out_host, sig_all_host);
}

int hbem_sv_dense_batch(int n, int nmat, unsigned d, const double* T_host, double* out_host, double* sig_all_host) {
    if (n < 2 || nmat < 1 || !T_host || !out_host || d > 2) return fail(HBEM_ERR_INVALID, "bad argument");
    HB_CK(cudaSetDevice(g_device));
    static thread_local DBuf T, A, V, out, status, sig;
    const size_t nn = (size_t)n * n, bytes = (size_t)nmat * (d + 1) * nn * sizeof(cplx);
    HB_CK(T.ensure(bytes));
    HB_CK(cudaMemcpy(T.p, T_host, bytes, cudaMemcpyHostToDevice));
    return sv_batch(0, n, nmat, d, T.as<cplx>(), (long long)((d + 1) * nn), (long long)nn, A, V, out, status, &sig,
                    out_host, sig_all_host);
}

int hbem_rand_sketch(int nr, int nc, unsigned long long seed, double* R_host) {
    if (nr < 1 || nc < 1 || !R_host) return fail(HBEM_ERR_INVALID, "rand_sketch: bad argument");
    std::mt19937_64 gen(seed);
    std::uniform_real_distribution<double> u(0., 1.);
    const double r = std::sqrt(0.5);
    for (size_t e = 0; e < (size_t)nr * nc; ++e) {
        R_host[2 * e] = u(gen) * r;
        R_host[2 * e + 1] = u(gen) * r;
    }
    return HBEM_OK;
}

int hbem_rsvd_sv_batch_device_ex(int n, int nmat, unsigned d, const void* T_dev, long long mat_stride,
                                 long long der_stride, const void* R_dev, int s, int q, int precision, int refine,
                                 double* out_host) {
    if (n < 2 || nmat < 1 || nmat > 65535 || d > 2 || !T_dev || !R_dev || !out_host || s < 1 || s > n || q < 0 ||
        precision < 0 || precision > 1 || refine < 1 || refine > 16)
        return fail(HBEM_ERR_INVALID, "rsvd_sv_batch: bad argument");
    if (!rsvd_supported(n, s, (int)d))
        return fail(HBEM_ERR_UNSUPPORTED, "rsvd_sv_batch: sketch wider than 32 columns, or a matrix too large for "
                                          "the shared-memory permutation buffer of the triangular solves");
    HB_CK(cudaSetDevice(g_device));
    static thread_local DBuf out, status, work;
    const size_t os = d + 1;
    HB_CK(out.ensure((size_t)nmat * os * sizeof(double)));
    HB_CK(status.ensure((size_t)nmat * sizeof(int)));
    const size_t wb = rsvd_work_bytes(n, nmat, s, (int)d, precision);
    HB_CK(work.ensure(std::max<size_t>(wb, 256)));
    long long nl = 0;
    HB_CK(rsvd_batched(n, nmat, s, q, (int)d, precision, refine, static_cast<const cplx*>(T_dev), mat_stride,
                       der_stride, static_cast<const cplx*>(R_dev), out.as<double>(), status.as<int>(), work.p,
                       work.cap, 0, &nl));
    g_launches += nl;
    std::vector<int> st(nmat);
    HB_CK(cudaMemcpy(out_host, out.p, (size_t)nmat * os * sizeof(double), cudaMemcpyDeviceToHost));
    HB_CK(cudaMemcpy(st.data(), status.p, (size_t)nmat * sizeof(int), cudaMemcpyDeviceToHost));
    for (int v : st)
        if (v == 4) return fail(HBEM_ERR_NOCONV, "rsvd_sv_batch: a tensor-core completion wait timed out");
        else if (v) return fail(HBEM_ERR_SINGULAR, "rsvd_sv_batch: zero pivot in the LU of T");
    return HBEM_OK;
}

int hbem_rsvd_sv_batch_device(int n, int nmat, unsigned d, const void* T_dev, long long mat_stride,
                              long long der_stride, const void* R_dev, int s, int q, double* out_host) {
    return hbem_rsvd_sv_batch_device_ex(n, nmat, d, T_dev, mat_stride, der_stride, R_dev, s, q, 0, 1, out_host);
}

int hbem_rsvd_sv_batch(int n, int nmat, unsigned d, const double* T_host, const double* R_host, int s, int q,
                       double* out_host) {
    if (n < 2 || nmat < 1 || d > 2 || !T_host || !R_host || !out_host || s < 1 || s > n)
        return fail(HBEM_ERR_INVALID, "rsvd_sv_batch: bad argument");
    HB_CK(cudaSetDevice(g_device));
    static thread_local DBuf T, R;
    const size_t nn = (size_t)n * n, bytes = (size_t)nmat * (d + 1) * nn * sizeof(cplx);
    HB_CK(T.ensure(bytes));
    HB_CK(R.ensure((size_t)n * s * sizeof(cplx)));
    HB_CK(cudaMemcpy(T.p, T_host, bytes, cudaMemcpyHostToDevice));
    HB_CK(cudaMemcpy(R.p, R_host, (size_t)n * s * sizeof(cplx), cudaMemcpyHostToDevice));
    return hbem_rsvd_sv_batch_device(n, nmat, d, T.p, (long long)((d + 1) * nn), (long long)nn, R.p, s, q, out_host);
}

int hbem_arnoldi_sv_batch_device(int n, int nmat, unsigned d, int count, double acc, const void* T_dev,
                                 long long mat_stride, long long der_stride, double* out_host, int* status_host,
                                 int* iters_host) {
    if (n < 2 || nmat < 1 || nmat > 65535 || d > 2 || count < 1 || count > n || !T_dev || !out_host ||
        !(acc >= 0.) || (long long)nmat * count > 65535)
        return fail(HBEM_ERR_INVALID, "arnoldi_sv_batch: bad argument");
    HB_CK(cudaSetDevice(g_device));
    // ARPACK takes tol <= 0 as machine precision; the FP64 residual of the block
    // iteration bottoms out near a few tens of eps
    const double tol = std::max(acc > 0. ? acc : kMachEps, 64. * kMachEps);
    const size_t os = d + 1, nout = (size_t)nmat * count * os;
    std::vector<int> stat(nmat, 0), iters(nmat, 0);
    if (arnoldi_supported(n, count, (int)d)) {
        static thread_local DBuf out, work;
        HB_CK(out.ensure(nout * sizeof(double)));
        HB_CK(work.ensure(std::max<size_t>(arnoldi_work_bytes(n, nmat, count, (int)d), 256)));
        long long nl = 0;
        HB_CK(arnoldi_batched(n, nmat, count, (int)d, tol, g_arnoldi_maxit, 0x5eedULL,
                              static_cast<const cplx*>(T_dev), mat_stride, der_stride, out.as<double>(), work.p,
                              work.cap, stat.data(), iters.data(), 0, &nl));
        g_launches += nl;
        HB_CK(cudaMemcpy(out_host, out.p, nout * sizeof(double), cudaMemcpyDeviceToHost));
    } else {
        // more singular values than the block holds: all n of them by the dense Jacobi
        // kernel, the count smallest kept (derivatives only through the block path)
        if (d > 0)
            return fail(HBEM_ERR_UNSUPPORTED, "arnoldi_sv_batch: derivatives need count <= 28 (block of 32 columns)");
        static thread_local DBuf A, V, out3, sdev, sig;
        std::vector<double> o3((size_t)nmat * 3), all((size_t)nmat * n);
        const int r = sv_batch(0, n, nmat, 0, static_cast<const cplx*>(T_dev), mat_stride, 0, A, V, out3, sdev, &sig,
                               o3.data(), all.data());
        if (r) return r;
        for (int m = 0; m < nmat; ++m) {
            std::sort(all.begin() + (size_t)m * n, all.begin() + (size_t)(m + 1) * n);
            for (int j = 0; j < count; ++j) out_host[(size_t)m * count + j] = all[(size_t)m * n + j];
        }
    }
    if (status_host) std::copy(stat.begin(), stat.end(), status_host);
    if (iters_host) std::copy(iters.begin(), iters.end(), iters_host);
    int worst = 0;
    for (int m = 0; m < nmat; ++m) {
        if (stat[m] == 5)
            for (size_t e = (size_t)m * count * os; e < (size_t)(m + 1) * count * os; ++e) out_host[e] = NAN;
        worst = std::max(worst, stat[m]);
    }
    if (worst == 5) return fail(HBEM_ERR_SINGULAR, "arnoldi_sv_batch: zero pivot in the LU of T");
    if (worst == 6) return fail(HBEM_ERR_NOCONV, "arnoldi_sv_batch: maximum number of iterations taken");
    return HBEM_OK;
}

int hbem_arnoldi_sv_batch(int n, int nmat, unsigned d, int count, double acc, const double* T_host,
                          double* out_host, int* status_host) {
    if (n < 2 || nmat < 1 || d > 2 || !T_host || !out_host) return fail(HBEM_ERR_INVALID, "arnoldi_sv_batch: bad argument");
    HB_CK(cudaSetDevice(g_device));
    static thread_local DBuf T;
    const size_t nn = (size_t)n * n, bytes = (size_t)nmat * (d + 1) * nn * sizeof(cplx);
    HB_CK(T.ensure(bytes));
    HB_CK(cudaMemcpy(T.p, T_host, bytes, cudaMemcpyHostToDevice));
    return hbem_arnoldi_sv_batch_device(n, nmat, d, count, acc, T.p, (long long)((d + 1) * nn), (long long)nn,
                                        out_host, status_host, nullptr);
}

int hbem_cgemm_f32_batch_device(int m, int n, int k, const void* A, long long lda, long long sa, const void* B,
                                long long ldb, long long sb, void* C, long long ldc, long long sc, int nmat,
                                int tensor_cores) {
    if (m < 0 || n < 0 || k < 0 || nmat < 1 || nmat > 65535 || !A || !B || !C || lda < std::max(1, m) ||
        ldb < std::max(1, k) || ldc < std::max(1, m))
        return fail(HBEM_ERR_INVALID, "cgemm_f32_batch: bad argument");
    HB_CK(cudaSetDevice(g_device));
    static thread_local DBuf err;
    HB_CK(err.ensure(sizeof(int)));
    HB_CK(cudaMemsetAsync(err.p, 0, sizeof(int), 0));
    HB_CK(launch_cgemm_f32(m, n, k, static_cast<const cplxf*>(A), lda, sa, static_cast<const cplxf*>(B), ldb, sb,
                           static_cast<cplxf*>(C), ldc, sc, nmat, tensor_cores, err.as<int>(), 0));
    g_launches += 1;
    int h = 0;
    HB_CK(cudaMemcpy(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h) return fail(HBEM_ERR_NOCONV, "cgemm_f32_batch: a tensor-core completion wait timed out");
    return HBEM_OK;
}

int hbem_lu_factor_batch_device_f32(int n, int nmat, void* A_dev, long long stride, int* piv_dev, int* info_host) {
    if (n < 1 || nmat < 1 || nmat > 65535 || !A_dev || !piv_dev || stride < (long long)n * n)
        return fail(HBEM_ERR_INVALID, "lu_factor_batch_f32: bad argument");
    if ((size_t)n * sizeof(int) > 220 * 1024) return fail(HBEM_ERR_UNSUPPORTED, "lu_factor_batch_f32: n too large");
    HB_CK(cudaSetDevice(g_device));
    static thread_local DBuf perm, info, tc_err;
    HB_CK(perm.ensure((size_t)nmat * n * sizeof(int)));
    HB_CK(info.ensure((size_t)nmat * sizeof(int)));
    HB_CK(tc_err.ensure(sizeof(int)));
    HB_CK(cudaMemsetAsync(tc_err.p, 0, sizeof(int), 0));
    long long nl = 0;
    HB_CK(lu_factor_batched_f32(n, nmat, static_cast<cplxf*>(A_dev), stride, piv_dev, perm.as<int>(), info.as<int>(),
                                0, &nl, tc_err.as<int>()));
    g_launches += nl;
    std::vector<int> inf(nmat);
    int terr = 0;
    HB_CK(cudaMemcpy(inf.data(), info.p, (size_t)nmat * sizeof(int), cudaMemcpyDeviceToHost));
    HB_CK(cudaMemcpy(&terr, tc_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (terr) return fail(HBEM_ERR_NOCONV, "lu_factor_batch_f32: a tensor-core completion wait timed out");
    int first = 0;
    for (int m = 0; m < nmat; ++m) {
        if (info_host) info_host[m] = inf[m];
        if (inf[m] && !first) first = m + 1;
    }
    if (first)
        return fail(HBEM_ERR_SINGULAR, "lu_factor_batch_f32: zero pivot (matrix " + std::to_string(first - 1) + ")");
    return HBEM_OK;
}

int hbem_lu_factor_batch_device(int n, int nmat, void* A_dev, long long stride, int* piv_dev, int* info_host) {
    if (n < 1 || nmat < 1 || nmat > 65535 || !A_dev || !piv_dev || stride < (long long)n * n)
        return fail(HBEM_ERR_INVALID, "lu_factor_batch: bad argument");
    if ((size_t)n * sizeof(int) > 220 * 1024) return fail(HBEM_ERR_UNSUPPORTED, "lu_factor_batch: n too large");
    HB_CK(cudaSetDevice(g_device));
    static thread_local DBuf perm, info;
    HB_CK(perm.ensure((size_t)nmat * n * sizeof(int)));
    HB_CK(info.ensure((size_t)nmat * sizeof(int)));
    long long nl = 0;
    HB_CK(lu_factor_batched(n, nmat, static_cast<cplx*>(A_dev), stride, piv_dev, perm.as<int>(), info.as<int>(), 0,
                            &nl));
    g_launches += nl;
    std::vector<int> inf(nmat);
    HB_CK(cudaMemcpy(inf.data(), info.p, (size_t)nmat * sizeof(int), cudaMemcpyDeviceToHost));
    int first = 0;
    for (int m = 0; m < nmat; ++m) {
        if (info_host) info_host[m] = inf[m];
        if (inf[m] && !first) first = m + 1;
    }
    if (first) return fail(HBEM_ERR_SINGULAR, "lu_factor_batch: zero pivot (matrix " + std::to_string(first - 1) + ")");
    return HBEM_OK;
}

int hbem_lu_solve_batch_device(int n, int nmat, int trans, const void* LU_dev, long long stride, const int* piv_dev,
                               int nrhs, void* X_dev, long long xstride) {
    if (n < 1 || nmat < 1 || nmat > 65535 || (trans != 0 && trans != 1) || !LU_dev || !piv_dev || nrhs < 1 ||
        !X_dev || stride < (long long)n * n || xstride < (long long)n * nrhs)
        return fail(HBEM_ERR_INVALID, "lu_solve_batch: bad argument");
    if (!lu_solve_supported(n)) return fail(HBEM_ERR_UNSUPPORTED, "lu_solve_batch: n too large");
    HB_CK(cudaSetDevice(g_device));
    static thread_local DBuf perm;
    HB_CK(perm.ensure((size_t)nmat * n * sizeof(int)));
    HB_CK(lu_perm_from_piv(n, nmat, piv_dev, perm.as<int>(), 0));
    HB_CK(lu_solve_batched(n, nmat, trans, static_cast<const cplx*>(LU_dev), stride, perm.as<int>(), nrhs,
                           static_cast<cplx*>(X_dev), xstride, 0));
    g_launches += 2;
    HB_CK(cudaStreamSynchronize(0));
    return HBEM_OK;
}

int hbem_solop_info(hbem_solop s, int* npanels) {
    if (!s || !npanels) return fail(HBEM_ERR_INVALID, "solop_info: bad argument");
    *npanels = s->b->n;
    return HBEM_OK;
}

int hbem_sigma_rsvd_sweep(hbem_solop s, const double* k_host, int nk, double c_o, double c_i, int sketch, int q,
                          int precision, unsigned long long seed, double* sigma_out) {
    if (!s || !k_host || !sigma_out || nk < 1 || sketch < 1 || q < 0 || precision < 0 || precision > 1)
        return fail(HBEM_ERR_INVALID, "sigma_rsvd_sweep: bad argument");
    hbem_builder b = s->b;
    HB_CK(cudaSetDevice(b->device));
    const int n = 2 * b->n;
    if (sketch > n) return fail(HBEM_ERR_INVALID, "sigma_rsvd_sweep: sketch wider than the matrix");
    const size_t mat = (size_t)n * n;
    static thread_local DBuf R;
    std::vector<double> Rh(2 * (size_t)n * sketch);
    if (int r = hbem_rand_sketch(n, sketch, seed, Rh.data())) return r;
    HB_CK(R.ensure(Rh.size() * sizeof(double)));
    HB_CK(cudaMemcpy(R.p, Rh.data(), Rh.size() * sizeof(double), cudaMemcpyHostToDevice));
    int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)nk, ((size_t)2 << 30) / (mat * sizeof(cplx))));
    chunk = std::min(chunk, 65535);
    HB_CK(s->d_T.ensure((size_t)chunk * mat * sizeof(cplx)));
    for (int k0 = 0; k0 < nk; k0 += chunk) {
        const int kn = std::min(chunk, nk - k0);
        if (int r = gen_T_batch(s, k_host + k0, nullptr, kn, c_o, c_i, 0, s->d_T.as<cplx>())) return r;
        HB_CK(cudaStreamSynchronize(b->st));
        if (int r = hbem_rsvd_sv_batch_device_ex(n, kn, 0, s->d_T.p, (long long)mat, (long long)mat, R.p, sketch, q,
                                                 precision, 3, sigma_out + k0))
            return r;
    }
    return HBEM_OK;
}

int hbem_sweep_sigma(hbem_solop s, const double* k_host, int nk, double c_o, double c_i, unsigned d, double* out_host) {
    if (!s || !k_host || !out_host || nk < 1 || d > 2) return fail(HBEM_ERR_INVALID, "bad argument");
    hbem_builder b = s->b;
    HB_CK(cudaSetDevice(b->device));
    const int n = 2 * b->n;
    const size_t mat = (size_t)n * n;
    // bound the T batch to ~2 GiB
    int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)nk, ((size_t)2 << 30) / ((d + 1) * mat * sizeof(cplx))));
    HB_CK(s->d_T.ensure((size_t)chunk * (d + 1) * mat * sizeof(cplx)));
    for (int k0 = 0; k0 < nk; k0 += chunk) {
        int kn = std::min(chunk, nk - k0);
        if (int r = gen_T_batch(s, k_host + k0, nullptr, kn, c_o, c_i, d, s->d_T.as<cplx>())) return r;
        if (int r = sv_batch(b->st, n, kn, d, s->d_T.as<cplx>(), (long long)(d + 1) * mat, (long long)mat, s->d_svdA,
                             s->d_svdV, s->d_out, s->d_status, nullptr, out_host + 3LL * k0, nullptr))
            return r;
    }
    return HBEM_OK;
}

// Many scatterers at once: every operator's T(k) batch and dense-SVD launch are
// enqueued on its own stream before any is waited for, so the small per-scatterer
// launches (one CTA per matrix in the SVD) run side by side on the GPU.
int hbem_sweep_sigma_multi(const hbem_solop* ops, int nops, const int* counts, const double* k_host,
                           const double* c_i_host, double c_o, unsigned d, double* out_host) {
    if (!ops || nops < 1 || !counts || !k_host || !c_i_host || !out_host || d > 2)
        return fail(HBEM_ERR_INVALID, "sweep_sigma_multi: bad argument");
    size_t total = 0;
    bool fast = svd_fast_on();
    for (int i = 0; i < nops; ++i) {
        if (!ops[i] || counts[i] < 0) return fail(HBEM_ERR_INVALID, "sweep_sigma_multi: bad argument");
        total += (size_t)counts[i];
        fast &= svd_fast_smem_bytes(2 * ops[i]->b->n) <= 220 * 1024;
    }
    if (!fast) {   // orders the fast kernel does not take: one operator after the other
        size_t off = 0;
        for (int i = 0; i < nops; ++i) {
            if (counts[i] > 0)
                if (int r = hbem_sweep_sigma(ops[i], k_host + off, counts[i], c_o, c_i_host[i], d, out_host + 3 * off))
                    return r;
            off += (size_t)counts[i];
        }
        return HBEM_OK;
    }
    static thread_local double* pin = nullptr;
    static thread_local size_t pin_cap = 0;
    const size_t need = total * 3 * sizeof(double) + total * sizeof(int);
    if (need > pin_cap) {
        if (pin) cudaFreeHost(pin);
        pin = nullptr;
        pin_cap = 0;
        HB_CK(cudaMallocHost(&pin, need));
        pin_cap = need;
    }
    int* pstat = reinterpret_cast<int*>(pin + total * 3);
    size_t off = 0;
    for (int i = 0; i < nops; ++i) {
        hbem_solop s = ops[i];
        const int kn = counts[i];
        if (kn > 0) {
            hbem_builder b = s->b;
            HB_CK(cudaSetDevice(b->device));
            const int n = 2 * b->n;
            const size_t mat = (size_t)n * n;
            HB_CK(s->d_T.ensure((size_t)kn * (d + 1) * mat * sizeof(cplx)));
            HB_CK(s->d_out.ensure((size_t)kn * 3 * sizeof(double)));
            HB_CK(s->d_status.ensure((size_t)kn * sizeof(int)));
            if (int r = gen_T_batch(s, k_host + off, nullptr, kn, c_o, c_i_host[i], d, s->d_T.as<cplx>())) return r;
            HB_CK(launch_svd_fast(n, kn, (int)d, s->d_T.as<cplx>(), (long long)(d + 1) * mat, (long long)mat,
                                  s->d_out.as<double>(), s->d_status.as<int>(), b->st));
            g_launches += 1;
            HB_CK(cudaMemcpyAsync(pin + 3 * off, s->d_out.p, (size_t)kn * 3 * sizeof(double), cudaMemcpyDeviceToHost,
                                  b->st));
            HB_CK(cudaMemcpyAsync(pstat + off, s->d_status.p, (size_t)kn * sizeof(int), cudaMemcpyDeviceToHost, b->st));
        }
        off += (size_t)kn;
    }
    for (int i = 0; i < nops; ++i)
        if (counts[i] > 0) HB_CK(cudaStreamSynchronize(ops[i]->b->st));
    std::copy(pin, pin + total * 3, out_host);
    // matrices the fast kernel could not finish: redone by the polished kernel
    off = 0;
    for (int i = 0; i < nops; ++i) {
        bool redo = g_svd_force_redo.load(std::memory_order_relaxed) != 0;
        for (int q = 0; q < counts[i]; ++q) redo |= pstat[off + q] != 0;
        if (redo) {
            const int save = t_svd_polished_only;
            t_svd_polished_only = 1;
            const int r = hbem_sweep_sigma(ops[i], k_host + off, counts[i], c_o, c_i_host[i], d, out_host + 3 * off);
            t_svd_polished_only = save;
            if (r) return r;
        }
        off += (size_t)counts[i];
    }
    return HBEM_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- accessors for other translation units

namespace hbem {

// host panel data and settings of a solutions operator's mesh
int solop_mesh(hbem_solop s, int* n, const int** kinds, const double** par, int* proj, int* device) {
    if (!s) return fail(HBEM_ERR_INVALID, "null solutions operator");
    if (!s->b->p1p1())
        return fail(HBEM_ERR_UNSUPPORTED, "the transmission problem needs P1 test and trial spaces (its traces are P1)");
    *n = s->b->n;
    *kinds = s->b->kind.data();
    *par = s->b->par.data();
    *proj = s->proj;
    *device = s->b->device;
    return HBEM_OK;
}

// T(k) of the operator (projected or not, as created) into T_dev (2N x 2N), synchronised
int solop_gen_T(hbem_solop s, double k_re, double k_im, double c_o, double c_i, void* T_dev) {
    if (int r = gen_T_batch(s, &k_re, &k_im, 1, c_o, c_i, 0, static_cast<cplx*>(T_dev))) return r;
    HB_CK(cudaStreamSynchronize(s->b->st));
    return HBEM_OK;
}

hbem_builder solop_builder(hbem_solop s) { return s ? s->b : nullptr; }

// Gauss-Legendre rule on [a, b] (getGaussQR, include/gauleg.hpp:35-79)
void gauss_rule(double a, double b, int n, double* x, double* w) { gauss_legendre(a, b, n, x, w); }

// launch counter shared by every entry point
void count_launches(long long n) { g_launches += n; }

// The plain search's Newton rounds add speculative bisection points where sigma comes
// from the one-CTA dense kernel (its per-evaluation latency, not the GPU's
// throughput, bounds a round, so a few more matrices per round cost little).
int plain_speculate_ok(hbem_solop s) {
    return s && g_plain_speculate && svd_fast_on() && svd_fast_smem_bytes(2 * s->b->n) <= 220 * 1024;
}

int plain_warm_start_ok() { return g_plain_warm_start; }

int plain_async_ok() { return g_plain_async; }
int plain_spec_limits(int* deep) {
    *deep = g_plain_spec_deep;
    return g_plain_spec_async;
}

// The FP32 V-set pool of the dense kernel's warm starts holds at least npool slots
// (contents kept when it grows).  Synchronous.
int vpool_ensure(hbem_solop s, int npool) {
    hbem_builder b = s->b;
    const size_t mat = 4ULL * b->n * b->n;
    const size_t pool_bytes = (size_t)npool * mat * sizeof(cplxf);
    if (pool_bytes <= s->d_vpool.cap) return HBEM_OK;
    HB_CK(cudaSetDevice(b->device));
    for (EvalLane* l : lane_pool(b->device).lanes) HB_CK(cudaStreamSynchronize(l->st));
    DBuf grown;
    HB_CK(grown.ensure(pool_bytes));
    if (s->d_vpool.p) {
        HB_CK(cudaMemcpyAsync(grown.p, s->d_vpool.p, s->d_vpool.cap, cudaMemcpyDeviceToDevice, b->st));
        HB_CK(cudaStreamSynchronize(b->st));
    }
    s->d_vpool.release();
    s->d_vpool = grown;
    return HBEM_OK;
}

// Lanes: asynchronous sigma and its first d derivatives (d = 1 or 2) of up to kLaneMaxPts wavenumbers
// through the one-CTA dense kernel with warm starts from the operator's pool (slots as
// sweep_sigma_warm).  lane_launch enqueues the assembly, the dense kernel and the copy
// of the results on the lane's own stream and returns; lane_wait tells whether the
// lane has finished (blocking when `block`); lane_results gives its values, redoing
// with the FP64-polished kernel, synchronously, any matrix the fast kernel could not
// finish.  The dense kernel must take the operator's order (plain_speculate_ok).
// the lanes up to `lane` of this thread's pool for `device` exist.  Lanes below
// kBulkLanes (the plain search's grid chunks) run at the lowest stream priority, lanes
// kBulkLanes .. kUrgentLanes - 1 (candidates deep into their Newton runs, the search's
// critical path) at the highest, the others (its other candidates' evaluations) one
// level above the lowest, so that a candidate's blocks are scheduled ahead of the
// grid's remaining ones and the longest runs' ahead of all.
constexpr int kBulkLanes = 8;
constexpr int kUrgentLanes = 16;
static int lane_make(int device, int lane) {
    std::vector<EvalLane*>& lanes = lane_pool(device).lanes;
    int least = 0, greatest = 0;
    HB_CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    while ((int)lanes.size() <= lane) {
        EvalLane* l = new EvalLane();
        lanes.push_back(l);
        const int idx = (int)lanes.size() - 1;
        const int mid = greatest < least - 1 ? least - 1 : greatest;
        const int prio = idx < kBulkLanes ? least : (idx < kUrgentLanes ? greatest : mid);
        HB_CK(cudaStreamCreateWithPriority(&l->st, cudaStreamNonBlocking, prio));
        HB_CK(cudaEventCreateWithFlags(&l->done, cudaEventDisableTiming));
        HB_CK(cudaEventCreateWithFlags(&l->asm_done, cudaEventDisableTiming));
        HB_CK(cudaMallocHost(&l->h_out, 3 * kLaneMaxPts * sizeof(double)));
        HB_CK(cudaMallocHost(&l->h_status, kLaneMaxPts * sizeof(int)));
    }
    return HBEM_OK;
}

int lane_launch(hbem_solop s, int lane, const double* k_host, int npts, double c_o, double c_i, const int* wslot,
                const int* oslot, int npool, unsigned d) {
    if (!s || lane < 0 || lane >= 64 || npts < 1 || npts > kLaneMaxPts || d > 2)
        return fail(HBEM_ERR_INVALID, "lane_launch: bad argument");
    hbem_builder b = s->b;
    HB_CK(cudaSetDevice(b->device));
    if (int r = lane_make(b->device, lane)) return r;
    std::vector<EvalLane*>& lanes = lane_pool(b->device).lanes;
    for (int i = 0; i < npts; ++i)
        if (wslot[i] >= npool || oslot[i] >= npool) return fail(HBEM_ERR_INVALID, "lane_launch: slot outside the pool");
    if (int r = vpool_ensure(s, npool)) return r;
    EvalLane& L = *lanes[lane];
    const int n = 2 * b->n;
    const size_t mat = (size_t)n * n;
    L.npts = npts;
    L.mode = 0;
    L.near_cur = false;
    std::copy(k_host, k_host + npts, L.k);
    std::vector<int> slots(2 * (size_t)npts);
    std::copy(wslot, wslot + npts, slots.begin());
    std::copy(oslot, oslot + npts, slots.begin() + npts);
    HB_CK(upload(L.slots, slots, L.st));
    L.d = (int)d;
    HB_CK(L.T.ensure((size_t)npts * (d + 1) * mat * sizeof(cplx)));
    HB_CK(L.out.ensure(3 * kLaneMaxPts * sizeof(double)));
    HB_CK(L.status.ensure(kLaneMaxPts * sizeof(int)));
    if (int r = gen_T_batch_ws(s, k_host, nullptr, npts, c_o, c_i, d, L.T.as<cplx>(), L.jobs, L.loc, L.st)) return r;
    HB_CK(launch_svd_fast(n, npts, (int)d, L.T.as<cplx>(), (long long)(d + 1) * (long long)mat, (long long)mat, L.out.as<double>(),
                          L.status.as<int>(), L.st, s->d_vpool.as<cplxf>(), L.slots.as<int>(), L.slots.as<int>() + npts,
                          nullptr));
    g_launches += 1;
    HB_CK(cudaMemcpyAsync(L.h_out, L.out.p, 3 * (size_t)npts * sizeof(double), cudaMemcpyDeviceToHost, L.st));
    HB_CK(cudaMemcpyAsync(L.h_status, L.status.p, (size_t)npts * sizeof(int), cudaMemcpyDeviceToHost, L.st));
    HB_CK(cudaEventRecord(L.done, L.st));
    return HBEM_OK;
}

void singular_split_hold(int on) { t_split_hold = on ? 1 : 0; }

// Points near the lane's last one without assembly: the lane has just evaluated one
// point with T, T', T'' (lane_launch with d = 2, or an earlier call of this one with
// d = 2); T, T' (and T'' for d = 2) at the npts (1 or 2) points k_host come from that
// point's three matrices by their Taylor polynomials (launch_taylor_near; each point
// within 1e-6 of it), then the dense kernel with warm slots wslot / oslot, all on the
// lane's own stream, behind the evaluation.  Uses: a root's two sign-change check
// points (d = 1) and a Newton step of at most 1e-6 (d = 2).  lane_results then gives
// the values as for lane_launch (a redo assembles the points).  HBEM_ERR_UNSUPPORTED
// when the lane holds no such point: the caller then assembles.
int lane_launch_near(hbem_solop s, int lane, const double* k_host, int npts, unsigned d, const int* wslot,
                     const int* oslot, int npool) {
    if (!s || lane < 0 || lane >= 64 || !k_host || !wslot || !oslot || npts < 1 || npts > 2 || d < 1 || d > 2)
        return fail(HBEM_ERR_INVALID, "lane_launch_near: bad argument");
    hbem_builder b = s->b;
    std::vector<EvalLane*>& lanes = lane_pool(b->device).lanes;
    if (lane >= (int)lanes.size()) return fail(HBEM_ERR_INVALID, "lane_launch_near: no such lane");
    EvalLane& L = *lanes[lane];
    if (L.mode != 0 || L.d != 2 || L.npts != 1) return HBEM_ERR_UNSUPPORTED;
    const double x = L.k[0];
    double h[2] = {0., 0.};
    for (int q = 0; q < npts; ++q) {
        h[q] = k_host[q] - x;
        if (!(std::fabs(h[q]) <= 1e-6)) return HBEM_ERR_UNSUPPORTED;
        if (wslot[q] >= npool || oslot[q] >= npool) return fail(HBEM_ERR_INVALID, "lane_launch_near: slot outside the pool");
    }
    HB_CK(cudaSetDevice(b->device));
    const int n = 2 * b->n;
    const size_t mat = (size_t)n * n;
    // the source point's matrices stay where they are; the new ones go to the other buffer
    DBuf& src = L.near_cur ? L.T2 : L.T;
    DBuf& dst = L.near_cur ? L.T : L.T2;
    if (dst.cap < (size_t)npts * (d + 1) * mat * sizeof(cplx)) {
        // growing a buffer drops its contents: only the destination may grow
        HB_CK(dst.ensure((size_t)npts * (d + 1) * mat * sizeof(cplx)));
    }
    L.npts = npts;
    L.d = (int)d;
    std::vector<int> slots(2 * (size_t)npts);
    for (int q = 0; q < npts; ++q) {
        L.k[q] = k_host[q];
        slots[q] = wslot[q];
        slots[npts + q] = oslot[q];
    }
    HB_CK(upload(L.slots, slots, L.st));
    HB_CK(launch_taylor_near((long long)mat, src.as<cplx>(), npts, h[0], h[1], (int)d, dst.as<cplx>(), L.st));
    HB_CK(launch_svd_fast(n, npts, (int)d, dst.as<cplx>(), (long long)(d + 1) * (long long)mat, (long long)mat,
                          L.out.as<double>(), L.status.as<int>(), L.st, s->d_vpool.as<cplxf>(), L.slots.as<int>(),
                          L.slots.as<int>() + npts, nullptr));
    L.near_cur = !L.near_cur;
    g_launches += 2;
    HB_CK(cudaMemcpyAsync(L.h_out, L.out.p, 3 * (size_t)npts * sizeof(double), cudaMemcpyDeviceToHost, L.st));
    HB_CK(cudaMemcpyAsync(L.h_status, L.status.p, (size_t)npts * sizeof(int), cudaMemcpyDeviceToHost, L.st));
    HB_CK(cudaEventRecord(L.done, L.st));
    return HBEM_OK;
}

int lane_wait(hbem_solop s, int lane, int block, int* finished) {
    EvalLane& L = *lane_pool(s->b->device).lanes[lane];
    cudaError_t e = block ? cudaEventSynchronize(L.done) : cudaEventQuery(L.done);
    if (e == cudaErrorNotReady) {
        *finished = 0;
        return HBEM_OK;
    }
    HB_CK(e);
    *finished = 1;
    return HBEM_OK;
}

// The plain search with its grid in chunks: the pool for `npool` V sets and room for
// the singular vectors of sigma_min at `npoints` grid points.  Synchronous.
int pipeline_setup(hbem_solop s, int npoints, int npool) {
    hbem_builder b = s->b;
    HB_CK(cudaSetDevice(b->device));
    if (int r = vpool_ensure(s, npool)) return r;
    const int n = 2 * b->n;
    s->uv_count = 0;
    HB_CK(s->d_uv.ensure((size_t)npoints * 2 * n * sizeof(cplx)));
    return HBEM_OK;
}

// the grid points have kept singular vectors (for sigma1_from_kept) up to npoints
void pipeline_keep_uv(hbem_solop s, int npoints) { s->uv_count = npoints; }

// Grid chunk on a lane: sigma at npts grid points first .. first + npts - 1 (cold
// start), the V sets to pool slots first + q and the singular vectors of sigma_min to
// rows first + q of the kept vectors.  The chunk's assembly starts after lane `after`'s
// assembly (-1: none), so chunks assemble in order while a chunk's dense kernel
// overlaps the next chunk's assembly.  lane_results then gives sigma (no redo:
// *all_fast = 0 when the fast kernel could not finish a matrix).
int lane_launch_grid(hbem_solop s, int lane, const double* k_host, int npts, int first, double c_o, double c_i,
                     int npool, int after) {
    if (!s || lane < 0 || lane >= 64 || npts < 1 || npts > kLaneMaxPts || first < 0 || first + npts > npool)
        return fail(HBEM_ERR_INVALID, "lane_launch_grid: bad argument");
    hbem_builder b = s->b;
    HB_CK(cudaSetDevice(b->device));
    if (int r = lane_make(b->device, std::max(lane, after))) return r;
    std::vector<EvalLane*>& lanes = lane_pool(b->device).lanes;
    EvalLane& L = *lanes[lane];
    const int n = 2 * b->n;
    const size_t mat = (size_t)n * n;
    L.npts = npts;
    L.mode = 1;
    L.d = 0;
    std::copy(k_host, k_host + npts, L.k);
    std::vector<int> slots(2 * (size_t)npts);
    for (int q = 0; q < npts; ++q) {
        slots[q] = -1;
        slots[npts + q] = first + q;
    }
    HB_CK(upload(L.slots, slots, L.st));
    HB_CK(L.T.ensure((size_t)npts * mat * sizeof(cplx)));
    HB_CK(L.out.ensure(3 * kLaneMaxPts * sizeof(double)));
    HB_CK(L.status.ensure(kLaneMaxPts * sizeof(int)));
    if (after >= 0) HB_CK(cudaStreamWaitEvent(L.st, lanes[after]->asm_done, 0));
    if (int r = gen_T_batch_ws(s, k_host, nullptr, npts, c_o, c_i, 0, L.T.as<cplx>(), L.jobs, L.loc, L.st)) return r;
    HB_CK(cudaEventRecord(L.asm_done, L.st));
    HB_CK(launch_svd_fast(n, npts, 0, L.T.as<cplx>(), (long long)mat, (long long)mat, L.out.as<double>(),
                          L.status.as<int>(), L.st, s->d_vpool.as<cplxf>(), L.slots.as<int>(), L.slots.as<int>() + npts,
                          s->d_uv.as<cplx>() + 2LL * n * first));
    g_launches += 1;
    HB_CK(cudaMemcpyAsync(L.h_out, L.out.p, 3 * (size_t)npts * sizeof(double), cudaMemcpyDeviceToHost, L.st));
    HB_CK(cudaMemcpyAsync(L.h_status, L.status.p, (size_t)npts * sizeof(int), cudaMemcpyDeviceToHost, L.st));
    HB_CK(cudaEventRecord(L.done, L.st));
    return HBEM_OK;
}

// Bracket ends on a lane: sigma' at two grid points from the grid's kept singular
// vectors (sigma1_from_kept for one candidate): T' assembled at k_host[0..1], then
// Re u^H T' v with (u, v) of grid points gidx[0..1].  lane_results gives sigma' in
// out_host[3q + 1].
int lane_launch_ends(hbem_solop s, int lane, const double* k_host, const int* gidx, double c_o, double c_i) {
    if (!s || lane < 0 || lane >= 64 || !k_host || !gidx) return fail(HBEM_ERR_INVALID, "lane_launch_ends: bad argument");
    hbem_builder b = s->b;
    HB_CK(cudaSetDevice(b->device));
    if (int r = lane_make(b->device, lane)) return r;
    EvalLane& L = *lane_pool(b->device).lanes[lane];
    const int n = 2 * b->n;
    const size_t mat = (size_t)n * n;
    L.npts = 2;
    L.mode = 2;
    L.d = 1;
    std::copy(k_host, k_host + 2, L.k);
    std::vector<int> id(gidx, gidx + 2);
    HB_CK(upload(L.slots, id, L.st));
    HB_CK(L.T.ensure(2 * 2 * mat * sizeof(cplx)));
    HB_CK(L.out.ensure(3 * kLaneMaxPts * sizeof(double)));
    if (int r = gen_T_batch_ws(s, k_host, nullptr, 2, c_o, c_i, 1, L.T.as<cplx>(), L.jobs, L.loc, L.st)) return r;
    HB_CK(launch_sigma1_uv(n, 2, L.T.as<cplx>() + mat, (long long)(2 * mat), s->d_uv.as<cplx>(), L.slots.as<int>(),
                           L.out.as<double>(), L.st));
    g_launches += 1;
    HB_CK(cudaMemcpyAsync(L.h_out, L.out.p, 2 * sizeof(double), cudaMemcpyDeviceToHost, L.st));
    HB_CK(cudaEventRecord(L.done, L.st));
    return HBEM_OK;
}

int lane_results_grid(hbem_solop s, int lane, double* sigma_host, int* all_fast) {
    EvalLane& L = *lane_pool(s->b->device).lanes[lane];
    *all_fast = 1;
    for (int i = 0; i < L.npts; ++i) {
        sigma_host[i] = L.h_out[3 * i];
        if (L.h_status[i] != 0) *all_fast = 0;
    }
    return HBEM_OK;
}

int lane_results_ends(hbem_solop s, int lane, double* d1_host) {
    EvalLane& L = *lane_pool(s->b->device).lanes[lane];
    d1_host[0] = L.h_out[0];
    d1_host[1] = L.h_out[1];
    return HBEM_OK;
}

int lane_results(hbem_solop s, int lane, double c_o, double c_i, double* out_host) {
    EvalLane& L = *lane_pool(s->b->device).lanes[lane];
    bool redo = g_svd_force_redo.load(std::memory_order_relaxed) != 0;
    for (int i = 0; i < L.npts; ++i) redo |= L.h_status[i] != 0;
    if (!redo) {
        std::copy(L.h_out, L.h_out + 3 * L.npts, out_host);
        return HBEM_OK;
    }
    const int save = t_svd_polished_only;
    t_svd_polished_only = 1;
    const int r = hbem_sweep_sigma(s, L.k, L.npts, c_o, c_i, (unsigned)L.d, out_host);
    t_svd_polished_only = save;
    return r;
}


// hbem_sweep_sigma through the one-CTA dense kernel with warm starts: a pool of npool
// FP32 V sets (2N x 2N each) held by the operator; wavenumber i starts its FP32
// Jacobi from slot warm_slot[i] and leaves its V set in slot out_slot[i] (-1: none).
// The pool's contents survive between calls while npool does not grow.  Returns
// HBEM_ERR_UNSUPPORTED when the dense kernel does not take the order or the batch.
int sweep_sigma_warm(hbem_solop s, const double* k_host, int nk, double c_o, double c_i, unsigned d,
                     const int* warm_slot, const int* out_slot, int npool, double* out_host, int keep_uv) {
    if (!s || !k_host || !out_host || nk < 1 || d > 2 || npool < 1 || !warm_slot || !out_slot)
        return fail(HBEM_ERR_INVALID, "sweep_sigma_warm: bad argument");
    hbem_builder b = s->b;
    const int n = 2 * b->n;
    const size_t mat = (size_t)n * n;
    if (!svd_fast_on() || svd_fast_smem_bytes(n) > 220 * 1024 || (size_t)nk * (d + 1) * mat * sizeof(cplx) > ((size_t)2 << 30))
        return fail(HBEM_ERR_UNSUPPORTED, "sweep_sigma_warm: the dense fast kernel does not take this batch");
    for (int i = 0; i < nk; ++i)
        if (warm_slot[i] >= npool || out_slot[i] >= npool)
            return fail(HBEM_ERR_INVALID, "sweep_sigma_warm: slot outside the pool");
    HB_CK(cudaSetDevice(b->device));
    const size_t pool_bytes = (size_t)npool * mat * sizeof(cplxf);
    if (pool_bytes > s->d_vpool.cap) {
        DBuf grown;
        HB_CK(grown.ensure(pool_bytes));
        if (s->d_vpool.p) {
            HB_CK(cudaMemcpyAsync(grown.p, s->d_vpool.p, s->d_vpool.cap, cudaMemcpyDeviceToDevice, b->st));
            HB_CK(cudaStreamSynchronize(b->st));
        }
        s->d_vpool.release();
        s->d_vpool = grown;
    }
    std::vector<int> slots(2 * (size_t)nk);
    std::copy(warm_slot, warm_slot + nk, slots.begin());
    std::copy(out_slot, out_slot + nk, slots.begin() + nk);
    HB_CK(upload(s->d_slots, slots, b->st));
    HB_CK(s->d_T.ensure((size_t)nk * (d + 1) * mat * sizeof(cplx)));
    if (int r = gen_T_batch(s, k_host, nullptr, nk, c_o, c_i, d, s->d_T.as<cplx>())) return r;
    if (keep_uv) {
        s->uv_count = 0;
        HB_CK(s->d_uv.ensure((size_t)nk * 2 * n * sizeof(cplx)));
    }
    int fast_ok = 0;
    if (int r = sv_batch(b->st, n, nk, d, s->d_T.as<cplx>(), (long long)(d + 1) * mat, (long long)mat, s->d_svdA,
                         s->d_svdV, s->d_out, s->d_status, nullptr, out_host, nullptr, s->d_vpool.as<cplxf>(),
                         s->d_slots.as<int>(), s->d_slots.as<int>() + nk, keep_uv ? s->d_uv.as<cplx>() : nullptr,
                         &fast_ok))
        return r;
    // the vectors are those of sigma only where the fast kernel's results were kept
    if (keep_uv && fast_ok) s->uv_count = nk;
    return HBEM_OK;
}

// sigma' at ne wavenumbers that an earlier sweep_sigma_warm(keep_uv) evaluated, from
// the singular vectors it kept: T and T' are assembled, then sigma' = Re u^H T' v
// (no second SVD; these are the same vectors up to rounding).  idx[e] is the position
// of wavenumber e in that sweep.  Returns HBEM_ERR_UNSUPPORTED when no vectors are kept.
int sigma1_from_kept(hbem_solop s, const double* k_host, const int* idx, int ne, double c_o, double c_i,
                     double* d1_host) {
    if (!s || !k_host || !idx || !d1_host || ne < 1) return fail(HBEM_ERR_INVALID, "sigma1_from_kept: bad argument");
    for (int e = 0; e < ne; ++e)
        if (idx[e] < 0 || idx[e] >= s->uv_count) return fail(HBEM_ERR_UNSUPPORTED, "sigma1_from_kept: no vectors");
    hbem_builder b = s->b;
    HB_CK(cudaSetDevice(b->device));
    const int n = 2 * b->n;
    const size_t mat = (size_t)n * n;
    HB_CK(s->d_T.ensure((size_t)ne * 2 * mat * sizeof(cplx)));
    if (int r = gen_T_batch(s, k_host, nullptr, ne, c_o, c_i, 1, s->d_T.as<cplx>())) return r;
    std::vector<int> id(idx, idx + ne);
    HB_CK(upload(s->d_slots, id, b->st));
    HB_CK(s->d_d1.ensure((size_t)ne * sizeof(double)));
    HB_CK(launch_sigma1_uv(n, ne, s->d_T.as<cplx>() + mat, (long long)(2 * mat), s->d_uv.as<cplx>(),
                           s->d_slots.as<int>(), s->d_d1.as<double>(), b->st));
    g_launches += 1;
    HB_CK(cudaMemcpyAsync(d1_host, s->d_d1.p, (size_t)ne * sizeof(double), cudaMemcpyDeviceToHost, b->st));
    HB_CK(cudaStreamSynchronize(b->st));
    return HBEM_OK;
}

}  // namespace hbem
