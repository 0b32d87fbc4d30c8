// runtime.cu -- host side of the C ABI in include/ggdmc_gpu.h.
//
// Owns device memory (a handle holds the design and the trials; a run adds
// chain state, proposal buffers and the sample store), builds one DE
// iteration as a launch sequence, captures a block of iterations into a CUDA
// graph and replays it, then copies the thinned samples back into the
// caller's arrays (R's posterior layout).
#include <algorithm>
#include <utility>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "../../include/ggdmc_gpu.h"
#include "sampler.cuh"

using namespace ggdmc;

namespace {

thread_local std::string g_err;
constexpr size_t kFlushBytes = (size_t)256 << 20;   // twice the 126 MB L2

ggdmc_status fail(ggdmc_status s, const std::string &msg)
{
    g_err = msg;
    return s;
}

#define CU(call)                                                                         \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess)                                                           \
            return fail(GGDMC_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

// Scratch for ggdmc_logprior_noalloc: one fixed array per device, so that
// entry point never allocates.  It holds the prior rows, then theta, then the
// output, each starting on a 256-byte boundary.
constexpr size_t kScratchDoubles = (size_t)1 << 17;   // 1 MiB
static __device__ __align__(256) double g_scratch[kScratchDoubles];

size_t round256(size_t n_double) { return (n_double + 31) & ~(size_t)31; }

// Device address of g_scratch in the current device's context, looked up on
// every call (cheap once the module is loaded; a cached address would not
// survive a device reset).  The first lookup on a device may load the module,
// so make the first call outside any stream capture.
ggdmc_status scratch_base(double **out)
{
    void *p = nullptr;
    CU(cudaGetSymbolAddress(&p, g_scratch));
    *out = static_cast<double *>(p);
    return GGDMC_OK;
}

template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t alloc(size_t count)
    {
        if (count <= n && p) return cudaSuccess;
        release();
        n = count;
        return cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
    }
    cudaError_t upload(const T *h, size_t count, cudaStream_t st)
    {
        cudaError_t e = alloc(count);
        if (e) return e;
        return count ? cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, st)
                     : cudaSuccess;
    }
};

// Page-locked host buffer (grows, kept by the handle across runs).
struct PinnedBuf {
    char *p = nullptr;
    size_t n = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf &) = delete;
    PinnedBuf &operator=(const PinnedBuf &) = delete;
    ~PinnedBuf() { release(); }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t alloc(size_t bytes)
    {
        if (bytes <= n && p) return cudaSuccess;
        release();
        n = bytes;
        return cudaHostAlloc((void **)&p, std::max<size_t>(bytes, 1), cudaHostAllocDefault);
    }
};

double host_Phi(double z) { return 0.5 * std::erfc(-z * 0.70710678118654752440); }

// Prior row (dist_id, p0, p1, lower, upper, c); see sampler.cuh.
ggdmc_status prior_rows(const ggdmc_prior *p, std::vector<double> &rows)
{
    if (!p || p->n_par <= 0 || !p->table) return fail(GGDMC_ERR_ARG, "prior table is empty");
    rows.assign((size_t)p->n_par * kPriorRow, 0.0);
    for (int j = 0; j < p->n_par; ++j) {
        const double *t = p->table + 6 * j;
        const int id = (int)t[4];
        if (t[5] == 0.0) return fail(GGDMC_ERR_ARG, "prior with log_p = FALSE is not supported");
        double *o = rows.data() + kPriorRow * j;
        o[0] = id; o[1] = t[0]; o[2] = t[1]; o[3] = t[2]; o[4] = t[3];
        if (id == GGDMC_PRIOR_TNORM) {
            const double mu = t[0], sg = t[1], lo = t[2], hi = t[3];
            if (!(sg > 0.0)) {
                o[5] = -INFINITY;
            } else {
                const double a = (lo - mu) / sg, b = (hi - mu) / sg;
                double mass;
                if (std::isinf(hi) && hi > 0) mass = 0.5 * std::erfc(a * 0.70710678118654752440);
                else if (std::isinf(lo) && lo < 0) mass = 0.5 * std::erfc(-b * 0.70710678118654752440);
                else mass = host_Phi(b) - host_Phi(a);
                o[5] = -0.91893853320467274178 - std::log(sg) - std::log(mass);
            }
        } else if (id == GGDMC_PRIOR_UNIF) {
            o[5] = -std::log(t[1] - t[0]);
        } else {
            return fail(GGDMC_ERR_ARG, "prior dist_id " + std::to_string(id) +
                                           " is not supported (1 = tnorm, 6 = unif)");
        }
    }
    return GGDMC_OK;
}

}  // namespace

// ------------------------------------------------------------------ handle
struct ggdmc_handle {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;       // the subject branch of a hierarchical sweep
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // design
    int model_type = 0, n_par = 0, n_cell = 0, n_acc = 0, n_ent = 0, n_const = 0, n_dent = 0;
    DevBuf<EntSrc> ent_src;
    DevBuf<uint8_t> cell_ent, cell_w, cell_t0;
    DevBuf<int32_t> t0_src, ddm_src;
    int n_t0 = 0;
    int n_sm = 0;
    DevBuf<double> consts;
    // trials
    int S = 0;
    int last_nmc = 0, last_C = 0, last_P = 0, last_Pphi = 0, last_S = 0;   // samples left by the last run
    std::vector<int64_t> h_offs;
    std::vector<int64_t> perm;     // stored trial j is data trial perm[j] (upload_data)
    DevBuf<int64_t> offs;
    DevBuf<double> rt64;
    DevBuf<float2> rt32;
    DevBuf<uint16_t> cell;
    // run workspace
    DevBuf<double> th, lp, ll, th_s, lp_s, ll_s, phi_tab, pp_bounds, prior, hprior, hrows;
    DevBuf<double> pth, plp, pll, pth_s, plp_s, pll_s, pref_src, pref_next;
    DevBuf<int32_t> partner, ptype, nstep, sub, migrated, ppartner, pptype, pnstep, psub,
        pmigrated, iter, status, items, items_plain, rs_para, sub_order, res_order, lvl_ns, ready, spec_cnt,
        ctl;
    DevBuf<int8_t> need, pneed;
    DevBuf<Ent32> tab_e;
    DevBuf<double> tab_lg;
    DevBuf<float2> tab_t;
    DevBuf<int32_t> cell_cnt;             // [S][n_cell] trials per subject and cell
    DevBuf<int32_t> tab_bad;
    DevBuf<double> jit, accu, pjit, paccu;
    DevBuf<double> smp_th, smp_lp, smp_ll, psmp_th, psmp_lp, psmp_ll, draws;
    DevBuf<unsigned long long> stats;
    DevBuf<double> io_a, io_b;
    DevBuf<Ent32> bt_e;                   // the likelihood batch's FP32 tables (k_batch_tables)
    DevBuf<double> bt_lg;
    DevBuf<float2> bt_t;
    DevBuf<int32_t> bt_bad;
    DevBuf<int32_t> ref_count, ref_base, ref_item;   // FP64 refinement of MIXED sums near zero
    DevBuf<double> ref_partial;
    DevBuf<uint8_t> flushbuf;
    PinnedBuf stage[2];                   // sample chunks on their way to the caller's buffers
    ggdmc_tuning tuning{};                // launch settings (0: built-in choice)

    DevModel dev_model() const
    {
        DevModel m{};
        m.model_type = model_type;
        m.n_par = n_par;
        m.n_cell = n_cell;
        m.n_acc = n_acc;
        m.n_ent = n_ent;
        m.n_const = n_const;
        m.n_t0 = n_t0;
        m.t0_src = t0_src.p;
        m.ent_src = ent_src.p;
        m.cell_ent = cell_ent.p;
        m.cell_w = cell_w.p;
        m.cell_t0 = cell_t0.p;
        m.ddm_src = ddm_src.p;
        m.n_dent = n_dent;
        m.consts = consts.p;
        return m;
    }
};

namespace {

double timeout_seconds()
{
    const char *s = std::getenv("GGDMC_TIMEOUT_S");
    double v = s ? std::atof(s) : 0.0;
    return v > 0.0 ? v : 1800.0;
}

// Wait for all work on the stream with a deadline; never blocks forever.
// Wait for an event with the GGDMC_TIMEOUT_S deadline (the host stops
// waiting; device work already queued still runs to its end).
ggdmc_status wait_event(cudaEvent_t ev)
{
    const auto t0 = std::chrono::steady_clock::now();
    const double lim = timeout_seconds();
    int spins = 0;
    for (;;) {
        const cudaError_t e = cudaEventQuery(ev);
        if (e == cudaSuccess) return GGDMC_OK;
        if (e != cudaErrorNotReady)
            return fail(GGDMC_ERR_CUDA, std::string("device work failed: ") + cudaGetErrorString(e));
        const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (el > lim) return fail(GGDMC_ERR_TIMEOUT, "device work exceeded GGDMC_TIMEOUT_S");
        if (++spins > 64) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

ggdmc_status wait_stream(cudaStream_t st)
{
    cudaEvent_t ev;
    CU(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, st);
    if (e) {
        cudaEventDestroy(ev);
        return fail(GGDMC_ERR_CUDA, std::string("cudaEventRecord: ") + cudaGetErrorString(e));
    }
    const ggdmc_status s = wait_event(ev);
    cudaEventDestroy(ev);
    return s;
}

// Diffusion model: two boundaries; the density of a cell depends only on the
// responding boundary's 8 parameters, so cells with equal (sources, boundary)
// share one entry.
ggdmc_status build_design_ddm(ggdmc_handle *h, const ggdmc_model *m)
{
    if (m->n_kind != GGDMC_DDM_NKIND) return fail(GGDMC_ERR_ARG, "DDM model needs n_kind == 8");
    if (m->n_acc != 2) return fail(GGDMC_ERR_ARG, "DDM model needs n_acc == 2 (two boundaries)");
    if (m->n_par < 1 || m->n_par > kMaxPar) return fail(GGDMC_ERR_ARG, "n_par out of range (1..64)");
    if (m->n_cell < 1 || m->n_cell > kMaxCell) return fail(GGDMC_ERR_ARG, "n_cell out of range");
    if (m->n_const < 0 || (m->n_const > 0 && !m->constants))
        return fail(GGDMC_ERR_ARG, "constants missing");
    std::map<std::vector<int32_t>, int> uniq;
    std::vector<int32_t> dsrc;
    std::vector<uint8_t> cent((size_t)m->n_cell * 2), cw(m->n_cell), ct0(m->n_cell, 0);
    for (int c = 0; c < m->n_cell; ++c) {
        const int w = m->resp[c];
        if (w < 0 || w > 1) return fail(GGDMC_ERR_ARG, "DDM resp must be 0 (lower) or 1 (upper)");
        std::vector<int32_t> key(m->param_src + ((size_t)c * 2 + w) * 8,
                                 m->param_src + ((size_t)c * 2 + w) * 8 + 8);
        for (int32_t q : key)
            if (!((q >= 0 && q < m->n_par) || (q < 0 && -1 - q < m->n_const)))
                return fail(GGDMC_ERR_ARG, "parameter source out of range");
        key.push_back(w);
        auto it = uniq.find(key);
        int id;
        if (it == uniq.end()) {
            id = (int)uniq.size();
            if (id >= kMaxDent) return fail(GGDMC_ERR_ARG, "too many distinct DDM cells");
            uniq[key] = id;
            dsrc.insert(dsrc.end(), key.begin(), key.end());
        } else {
            id = it->second;
        }
        cent[(size_t)c * 2] = cent[(size_t)c * 2 + 1] = (uint8_t)id;
        cw[c] = (uint8_t)w;
    }
    h->model_type = GGDMC_MODEL_DDM;
    h->n_par = m->n_par;
    h->n_cell = m->n_cell;
    h->n_acc = 2;
    h->n_ent = 0;
    h->n_t0 = 0;
    h->n_dent = (int)uniq.size();
    h->n_const = m->n_const;
    std::vector<double> consts(m->constants, m->constants + m->n_const);
    if (consts.empty()) consts.push_back(0.0);
    cudaStream_t st = h->stream;
    CU(h->ddm_src.upload(dsrc.data(), dsrc.size(), st));
    CU(h->cell_ent.upload(cent.data(), cent.size(), st));
    CU(h->cell_w.upload(cw.data(), cw.size(), st));
    CU(h->cell_t0.upload(ct0.data(), ct0.size(), st));
    CU(h->consts.upload(consts.data(), consts.size(), st));
    CU(configure_kernels(h->dev_model()));
    return GGDMC_OK;
}

ggdmc_status build_design(ggdmc_handle *h, const ggdmc_model *m)
{
    if (!m || !m->param_src || !m->resp) return fail(GGDMC_ERR_ARG, "model is NULL or incomplete");
    if (m->model_type == GGDMC_MODEL_DDM) return build_design_ddm(h, m);
    if (m->model_type != GGDMC_MODEL_LBA) return fail(GGDMC_ERR_ARG, "unknown model_type");
    if (m->n_kind != GGDMC_LBA_NKIND) return fail(GGDMC_ERR_ARG, "LBA model needs n_kind == 6");
    if (m->n_par < 1 || m->n_par > kMaxPar) return fail(GGDMC_ERR_ARG, "n_par out of range (1..64)");
    if (m->n_cell < 1 || m->n_cell > kMaxCell) return fail(GGDMC_ERR_ARG, "n_cell out of range");
    if (m->n_acc < 2 || m->n_acc > kMaxAcc) return fail(GGDMC_ERR_ARG, "n_acc out of range (2..8)");
    if (m->n_const < 0 || (m->n_const > 0 && !m->constants))
        return fail(GGDMC_ERR_ARG, "constants missing");
    auto check_src = [&](int32_t s) {
        return (s >= 0 && s < m->n_par) || (s < 0 && -1 - s < m->n_const);
    };
    auto value_if_const = [&](int32_t s, double &v) {
        if (s < 0) { v = m->constants[-1 - s]; return true; }
        return false;
    };
    const int K = m->n_acc, NK = m->n_kind;
    std::map<std::tuple<int, int, int, int>, int> uniq;
    std::vector<EntSrc> ents;
    std::vector<uint8_t> cent((size_t)m->n_cell * K), cw(m->n_cell);
    std::vector<int32_t> ct0(m->n_cell);
    std::vector<uint8_t> ct0i(m->n_cell);
    std::vector<int32_t> t0s;
    for (int c = 0; c < m->n_cell; ++c) {
        if (m->resp[c] < 0 || m->resp[c] >= K) return fail(GGDMC_ERR_ARG, "resp index out of range");
        // entries winner first, then the other accumulators in order (the
        // order of the survivor product is kept)
        cw[c] = 0;
        for (int kk = 0; kk < K; ++kk) {
            const int k = (kk == 0) ? m->resp[c] : (kk <= m->resp[c] ? kk - 1 : kk);
            const int32_t *q = m->param_src + ((size_t)c * K + k) * NK;
            for (int j = 0; j < NK; ++j)
                if (!check_src(q[j])) return fail(GGDMC_ERR_ARG, "parameter source out of range");
            double st0;
            if (!value_if_const(q[5], st0) || st0 != 0.0)
                return fail(GGDMC_ERR_ARG, "LBA with st0 other than the constant 0 is not supported");
            if (kk == 0) ct0[c] = q[4];
            else if (q[4] != ct0[c])
                return fail(GGDMC_ERR_ARG, "t0 must be the same for every accumulator of a cell");
            auto key = std::make_tuple(q[0], q[1], q[2], q[3]);
            auto it = uniq.find(key);
            int id;
            if (it == uniq.end()) {
                id = (int)ents.size();
                if (id >= kMaxEnt) return fail(GGDMC_ERR_ARG, "too many distinct accumulator tuples");
                uniq[key] = id;
                ents.push_back(EntSrc{q[0], q[1], q[2], q[3]});
            } else {
                id = it->second;
            }
            cent[(size_t)c * K + kk] = (uint8_t)id;
        }
    }
    for (int c = 0; c < m->n_cell; ++c) {
        auto it = std::find(t0s.begin(), t0s.end(), ct0[c]);
        if (it == t0s.end()) {
            if ((int)t0s.size() >= kMaxT0) return fail(GGDMC_ERR_ARG, "too many distinct t0 sources");
            t0s.push_back(ct0[c]);
            it = t0s.end() - 1;
        }
        ct0i[c] = (uint8_t)(it - t0s.begin());
    }
    h->n_t0 = (int)t0s.size();
    h->model_type = m->model_type;
    h->n_par = m->n_par;
    h->n_cell = m->n_cell;
    h->n_acc = K;
    h->n_ent = (int)ents.size();
    h->n_const = m->n_const;
    std::vector<double> consts(m->constants, m->constants + m->n_const);
    if (consts.empty()) consts.push_back(0.0);
    cudaStream_t st = h->stream;
    CU(h->ent_src.upload(ents.data(), ents.size(), st));
    CU(h->cell_ent.upload(cent.data(), cent.size(), st));
    CU(h->cell_w.upload(cw.data(), cw.size(), st));
    CU(h->cell_t0.upload(ct0i.data(), ct0i.size(), st));
    CU(h->t0_src.upload(t0s.data(), t0s.size(), st));
    CU(h->consts.upload(consts.data(), consts.size(), st));
    CU(configure_kernels(h->dev_model()));
    return GGDMC_OK;
}

ggdmc_status upload_data(ggdmc_handle *h, const ggdmc_data *d)
{
    if (!d) { h->S = 0; h->h_offs.assign(1, 0); return GGDMC_OK; }
    if (d->n_subject < 0 || !d->offsets) return fail(GGDMC_ERR_ARG, "data is incomplete");
    const int S = d->n_subject;
    std::vector<int64_t> offs(d->offsets, d->offsets + S + 1);
    if (offs[0] != 0) return fail(GGDMC_ERR_ARG, "offsets[0] must be 0");
    for (int s = 0; s < S; ++s)
        if (offs[s + 1] < offs[s]) return fail(GGDMC_ERR_ARG, "offsets must be non-decreasing");
    const int64_t N = offs[S];
    if (N > 0 && (!d->rt || !d->cell)) return fail(GGDMC_ERR_ARG, "rt / cell missing");
    std::vector<int32_t> cnt((size_t)std::max(S, 1) * h->n_cell, 0);
    for (int64_t i = 0; i < N; ++i) {
        if (!std::isfinite(d->rt[i])) return fail(GGDMC_ERR_ARG, "non-finite RT in data");
        if (d->cell[i] < 0 || d->cell[i] >= h->n_cell) return fail(GGDMC_ERR_ARG, "cell index out of range");
    }
    // Each subject's trials are stored by (cell, RT): a warp's 32 trials then
    // mostly share a cell (one table entry set, read as a shared-memory
    // broadcast) and a response-time range (the same branches of the FP32
    // density).  A subject's sums do not depend on the order beyond
    // rounding; perm maps a stored trial back to its place in the data.
    std::vector<int64_t> perm(N);
    std::vector<double> r64(N);
    std::vector<uint16_t> c16(N);
    // subjects in blocks over host threads (each writes only its subjects'
    // ranges of perm, cnt, r64 and c16)
    auto sort_subjects = [&](int s0, int s1) {
        std::vector<int64_t> pos(h->n_cell);
        std::vector<std::pair<double, int64_t>> seg;
        for (int s = s0; s < s1; ++s) {
            int32_t *cs = cnt.data() + (size_t)s * h->n_cell;
            for (int64_t i = offs[s]; i < offs[s + 1]; ++i) ++cs[d->cell[i]];
            int64_t at = offs[s];
            for (int c = 0; c < h->n_cell; ++c) {
                pos[c] = at;
                at += cs[c];
            }
            for (int64_t i = offs[s]; i < offs[s + 1]; ++i) perm[pos[d->cell[i]]++] = i;   // by cell, stable
            for (int c = 0, b = 0; c < h->n_cell; b += cs[c], ++c) {
                if (cs[c] < 2) continue;
                int64_t *q = perm.data() + offs[s] + b;
                seg.resize(cs[c]);
                for (int j = 0; j < cs[c]; ++j) seg[j] = {d->rt[q[j]], q[j]};
                std::sort(seg.begin(), seg.end());     // by RT, then data order
                for (int j = 0; j < cs[c]; ++j) q[j] = seg[j].second;
            }
            for (int64_t j = offs[s]; j < offs[s + 1]; ++j) {
                r64[j] = d->rt[perm[j]];
                c16[j] = (uint16_t)d->cell[perm[j]];
            }
        }
    };
    const int nt = (int)std::min<int64_t>({(int64_t)std::max(1u, std::thread::hardware_concurrency()), 16,
                                           (int64_t)std::max(S, 1), std::max<int64_t>(1, N / 20000)});
    if (nt <= 1) {
        sort_subjects(0, S);
    } else {
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t) pool.emplace_back(sort_subjects, (int)((int64_t)S * t / nt), (int)((int64_t)S * (t + 1) / nt));
        for (auto &th : pool) th.join();
    }
    h->S = S;
    h->h_offs = offs;
    h->perm = std::move(perm);
    cudaStream_t st = h->stream;
    CU(h->offs.upload(offs.data(), offs.size(), st));
    CU(h->rt64.upload(r64.data(), N, st));
    CU(h->rt32.alloc(N));
    CU(launch_split_rt(h->rt64.p, N, h->rt32.p, st));     // (hi, lo) FP32 pairs on the device
    CU(h->cell.upload(c16.data(), N, st));
    CU(h->cell_cnt.upload(cnt.data(), cnt.size(), st));
    return wait_stream(st);
}

ggdmc_status check_cfg(const ggdmc_de_config *c)
{
    if (!c) return fail(GGDMC_ERR_ARG, "config is NULL");
    if (c->nchain <= 2) return fail(GGDMC_ERR_ARG, "Require three or more chains.");
    if (c->nchain > kMaxChain) return fail(GGDMC_ERR_ARG, "nchain above 1024");
    if (c->nmc < 1 || c->thin < 1) return fail(GGDMC_ERR_ARG, "nmc and thin must be >= 1");
    if ((int64_t)(c->nmc - 1) * c->thin > INT32_MAX - 1)
        return fail(GGDMC_ERR_ARG, "(nmc - 1) * thin iterations exceed the 32-bit iteration counter");
    if (c->nparameter < 1 || c->nparameter > kMaxTheta)
        return fail(GGDMC_ERR_ARG, "nparameter out of range");
    if (!(c->rp > 0.0) || !(c->gamma_precursor > 0.0))
        return fail(GGDMC_ERR_ARG, "rp and gamma_precursor must be positive");
    if (c->precision < GGDMC_FP64 || c->precision > GGDMC_FP64_PLAIN)
        return fail(GGDMC_ERR_ARG, "unknown precision");
    return GGDMC_OK;
}

enum RunKind { RK_SUBJECTS, RK_HIER, RK_HYPER };

struct RunArgs {
    RunKind kind;
    const ggdmc_de_config *cfg;
    const ggdmc_prior *p_prior, *h_prior;
    ggdmc_chain_state *phi_state, *subj_state;
    const double *draws;
    ggdmc_samples *phi_out, *subj_out;
    ggdmc_run_stats *stats;
    const double *hyper_rows;
    int n_row;
};

static double ms_since(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

ggdmc_status run_impl(ggdmc_handle *h, const RunArgs &a)
{
    const auto t_in = std::chrono::steady_clock::now();
    double t_setup = 0.0, t_capture = 0.0, t_run = 0.0;
    ggdmc_status s;
    if ((s = check_cfg(a.cfg))) return s;
    const ggdmc_de_config &c = *a.cfg;
    const int C = c.nchain;
    const bool hier = a.kind == RK_HIER;
    const bool hyper = a.kind == RK_HYPER;
    const int S = hyper ? 0 : h->S;
    const int P = hyper ? 0 : h->n_par;
    int Pphi = 0;
    std::vector<double> prow, hrow, bounds;
    if ((s = prior_rows(a.p_prior, prow))) return s;
    if (hier || hyper) {
        if (!a.h_prior) return fail(GGDMC_ERR_ARG, "h_prior is required");
        if ((s = prior_rows(a.h_prior, hrow))) return s;
        Pphi = a.h_prior->n_par;
        if (Pphi != 2 * a.p_prior->n_par)
            return fail(GGDMC_ERR_ARG, "h_prior must have twice the parameters of p_prior");
        if (Pphi > kMaxTheta) return fail(GGDMC_ERR_ARG, "phi has too many parameters");
        if (!a.phi_state) return fail(GGDMC_ERR_ARG, "phi state is required");
        bounds.resize(2 * (size_t)a.p_prior->n_par);
        for (int j = 0; j < a.p_prior->n_par; ++j) {
            bounds[2 * j] = a.p_prior->table[6 * j + 2];
            bounds[2 * j + 1] = a.p_prior->table[6 * j + 3];
        }
    }
    if (!hyper) {
        if (S < 1) return fail(GGDMC_ERR_ARG, "no subjects in the handle");
        if (a.p_prior->n_par != P) return fail(GGDMC_ERR_ARG, "p_prior size differs from n_par");
        if (!a.subj_state) return fail(GGDMC_ERR_ARG, "subject state is required");
        if (!hier && c.nparameter != P)
            return fail(GGDMC_ERR_ARG, "nparameter must equal the model's n_par");
        if (hier && c.nparameter / 2 > P)
            return fail(GGDMC_ERR_ARG, "nparameter/2 exceeds the subject parameters");
    } else if (c.nparameter > Pphi) {
        return fail(GGDMC_ERR_ARG, "nparameter exceeds the phi parameters");
    }
    if (hier && c.nparameter > Pphi) return fail(GGDMC_ERR_ARG, "nparameter exceeds phi length");

    cudaStream_t st = h->stream;
    const int nmc = c.nmc;
    const int64_t n_iter = (int64_t)(nmc - 1) * c.thin;
    const int n_level = hier ? S + 1 : (hyper ? 1 : S);
    int64_t n_pass_draw = 1;
    if (hier) n_pass_draw = std::max<int64_t>(c.is_hblocked ? c.nparameter : 1,
                                              c.is_pblocked ? c.nparameter / 2 : 1);
    else if (c.is_pblocked) n_pass_draw = c.nparameter;
    const int64_t n_slot = GGDMC_DRAW_SLOTS(C, c.nparameter);

    // ---- device buffers
    const int CS = 2 * C;   // speculative proposals, then migration variants
    // Proposals per speculative work item (one pass over the subject's
    // trials).  Smaller items balance the launch better.  The 4-accumulator
    // LBA measured fastest at 2 (0.584 ms per sweep against 0.604 at 1 and
    // 0.595 at 4), the diffusion model and the 2-accumulator fits at 1
    // (hier_ddm_64 2.34 / 2.43 / 3.10 ms, many_fits_1024 3.44 / 3.75 / 4.56 ms).
    int spec_group = (h->model_type == GGDMC_MODEL_DDM || h->n_acc < 4) ? 1 : 2;
    if (h->tuning.spec_group > 0) spec_group = std::min(4, h->tuning.spec_group);
    if (const char *gs = std::getenv("GGDMC_SPEC_GROUP")) spec_group = std::min(4, std::max(1, std::atoi(gs)));
    int n_spec_items = 0;
    if (S > 0) {
        CU(h->th.alloc((size_t)S * C * P));
        CU(h->lp.alloc((size_t)S * C));
        CU(h->ll.alloc((size_t)S * C));
        CU(h->th_s.alloc((size_t)S * CS * P));
        CU(h->lp_s.alloc((size_t)S * CS));
        CU(h->ll_s.alloc((size_t)S * CS));
        CU(h->partner.alloc((size_t)S * C * 2));
        CU(h->need.alloc((size_t)S * CS));
        CU(h->ptype.alloc(S));
        CU(h->nstep.alloc(S));
        CU(h->sub.alloc((size_t)S * C));
        CU(h->migrated.alloc(S));
        CU(h->jit.alloc((size_t)S * C * P));
        CU(h->accu.alloc((size_t)S * C));
        CU(h->rs_para.alloc(S));
        CU(h->tab_e.alloc((size_t)S * CS * h->n_ent));
        CU(h->tab_lg.alloc((size_t)S * CS * h->n_ent));
        CU(h->tab_t.alloc((size_t)S * CS * h->n_t0));
        CU(h->tab_bad.alloc((size_t)S * CS));
        CU(h->smp_th.alloc((size_t)S * nmc * C * P));
        CU(h->smp_lp.alloc((size_t)S * nmc * C));
        CU(h->smp_ll.alloc((size_t)S * nmc * C));
        std::vector<double> buf((size_t)S * C * P), b1((size_t)S * C), b2((size_t)S * C);
        for (int l = 0; l < S; ++l) {
            const ggdmc_chain_state &cs = a.subj_state[l];
            if (!cs.theta || !cs.lp || !cs.ll) return fail(GGDMC_ERR_ARG, "subject state incomplete");
            std::memcpy(buf.data() + (size_t)l * C * P, cs.theta, sizeof(double) * C * P);
            std::memcpy(b1.data() + (size_t)l * C, cs.lp, sizeof(double) * C);
            std::memcpy(b2.data() + (size_t)l * C, cs.ll, sizeof(double) * C);
        }
        CU(cudaMemcpyAsync(h->th.p, buf.data(), sizeof(double) * buf.size(), cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(h->lp.p, b1.data(), sizeof(double) * b1.size(), cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(h->ll.p, b2.data(), sizeof(double) * b2.size(), cudaMemcpyHostToDevice, st));
        { ggdmc_status ws_ = wait_stream(st); if (ws_) return ws_; }
        // trial-count-descending work list for the likelihood kernel
        std::vector<int> order(S);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
            return (h->h_offs[x + 1] - h->h_offs[x]) > (h->h_offs[y + 1] - h->h_offs[y]);
        });
        std::vector<int32_t> items, plain((size_t)S * CS);
        for (int q = 0; q < S; ++q) {
            for (int k = 0; k < C; k += spec_group) items.push_back(order[q] * CS + k);
            for (int k = C; k < CS; k += spec_group) items.push_back(order[q] * CS + k);
        }
        n_spec_items = (int)items.size();
        for (size_t q = 0; q < plain.size(); ++q) plain[q] = (int32_t)q;
        CU(h->items.upload(items.data(), items.size(), st));
        CU(h->items_plain.upload(plain.data(), plain.size(), st));
        CU(h->sub_order.upload(order.data(), order.size(), st));
        CU(h->res_order.upload(order.data(), order.size(), st));
        CU(h->lvl_ns.alloc(S));
        CU(cudaMemsetAsync(h->lvl_ns.p, 0, sizeof(int32_t) * S, st));
    }
    if (Pphi > 0) {
        CU(h->pth.alloc((size_t)C * Pphi));
        CU(h->plp.alloc(C));
        CU(h->pll.alloc(C));
        CU(h->pth_s.alloc((size_t)C * Pphi));
        CU(h->plp_s.alloc(C));
        CU(h->pll_s.alloc(C));
        CU(h->pref_src.alloc(C));
        CU(h->pref_next.alloc(C));
        CU(h->ppartner.alloc((size_t)C * 2));
        CU(h->pneed.alloc(C));
        CU(h->pptype.alloc(1));
        CU(h->pnstep.alloc(1));
        CU(h->psub.alloc(C));
        CU(h->pmigrated.alloc(1));
        CU(h->pjit.alloc((size_t)C * Pphi));
        CU(h->paccu.alloc(C));
        CU(h->psmp_th.alloc((size_t)nmc * C * Pphi));
        CU(h->psmp_lp.alloc((size_t)nmc * C));
        CU(h->psmp_ll.alloc((size_t)nmc * C));
        CU(h->hprior.upload(hrow.data(), hrow.size(), st));
        CU(h->pp_bounds.upload(bounds.data(), bounds.size(), st));
        const ggdmc_chain_state &ps = *a.phi_state;
        if (!ps.theta || !ps.lp || !ps.ll) return fail(GGDMC_ERR_ARG, "phi state incomplete");
        CU(cudaMemcpyAsync(h->pth.p, ps.theta, sizeof(double) * C * Pphi, cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(h->plp.p, ps.lp, sizeof(double) * C, cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(h->pll.p, ps.ll, sizeof(double) * C, cudaMemcpyHostToDevice, st));
    }
    if (hier) CU(h->phi_tab.alloc((size_t)C * P * 3));
    if (!hier && !hyper) CU(h->prior.upload(prow.data(), prow.size(), st));
    if (hyper) {
        if (!a.hyper_rows || a.n_row < 1) return fail(GGDMC_ERR_ARG, "hyper data is empty");
        CU(h->hrows.upload(a.hyper_rows, (size_t)a.n_row * (Pphi / 2), st));
    }
    const int64_t n_draw = n_iter * n_level * n_pass_draw * n_slot;
    if (a.draws) CU(h->draws.upload(a.draws, (size_t)n_draw, st));
    const bool plain = c.precision == GGDMC_FP64_PLAIN;
    CU(h->iter.alloc(1));
    CU(h->status.alloc(1));
    CU(h->stats.alloc(ST_N));
    CU(cudaMemsetAsync(h->stats.p, 0, sizeof(unsigned long long) * ST_N, st));
    CU(cudaMemsetAsync(h->iter.p, 0, sizeof(int32_t), st));
    CU(cudaMemsetAsync(h->status.p, 0, sizeof(int32_t), st));
    // The subject pass fused with the next iteration's proposals
    // (k_sub_step) needs one subject pass per iteration and not the plain
    // form.  It pays where the levels come in more than one wave: the next
    // iteration's proposals and evaluations then fill the SMs the ordered
    // decisions leave idle.  Many independent fits: from two waves per SM.
    // Hierarchical: from one wave (the 256-subject workload: 0.823 ms per
    // sweep against 0.844 for the ordered resolve); the rest of the
    // speculative evaluations runs beside the phi update of t + 1.
    // GGDMC_FUSED=0/1 overrides the choice.
    const int sub_npass = hier ? (c.is_pblocked ? c.nparameter / 2 : 1) : (c.is_pblocked ? c.nparameter : 1);
    const bool fusable = S > 0 && !plain && sub_npass == 1;
    bool fused = fusable && (hier ? S > h->n_sm : (Pphi == 0 && S >= 2 * h->n_sm));
    if (const char *fs = std::getenv("GGDMC_FUSED")) fused = fusable && std::atoi(fs) != 0;
    if (fused) {
        CU(h->ready.alloc(S));
        CU(h->spec_cnt.alloc(S));
        CU(h->ctl.alloc(3));
        CU(cudaMemsetAsync(h->ready.p, 0xff, sizeof(int32_t) * S, st));   // -1: no iteration

        CU(cudaMemsetAsync(h->spec_cnt.p, 0, sizeof(int32_t) * S, st));
        CU(cudaMemsetAsync(h->ctl.p, 0, sizeof(int32_t) * 3, st));
    }

    // ---- run description
    RunDev r{};
    r.C = C; r.P = P; r.Pphi = Pphi; r.S = S;
    r.Pn = c.nparameter; r.half = c.nparameter / 2;
    r.loop = hier ? LOOP_HCHAINS : LOOP_CHAINS;
    r.level0 = hier ? 1 : 0;
    r.prec = (c.precision == GGDMC_MIXED) ? PREC_MIXED : PREC_FP64;
    r.sub_blocked = c.is_pblocked;
    r.phi_blocked = hier ? c.is_hblocked : c.is_pblocked;
    r.phi_loop = hier ? LOOP_HCHAINS : LOOP_CHAINS;
    r.thin = c.thin; r.nmc = nmc;
    r.gamma = c.gamma_precursor / std::sqrt(2.0 * c.nparameter);
    r.rp = c.rp; r.sub_mig = c.sub_migration_prob; r.pop_mig = c.pop_migration_prob;
    r.ds.draws = a.draws ? h->draws.p : nullptr;
    r.ds.seed = c.seed;
    r.ds.n_level = n_level; r.ds.n_pass = n_pass_draw; r.ds.n_slot = n_slot;
    r.iter = h->iter.p;
    r.m = h->dev_model();
    r.offs = h->offs.p; r.rt64 = h->rt64.p; r.rt32 = h->rt32.p; r.cell = h->cell.p;
    r.th = h->th.p; r.lp = h->lp.p; r.ll = h->ll.p;
    r.th_s = h->th_s.p; r.lp_s = h->lp_s.p; r.ll_s = h->ll_s.p;
    r.partner = h->partner.p; r.need = h->need.p; r.ptype = h->ptype.p; r.nstep = h->nstep.p;
    r.sub = h->sub.p; r.migrated = h->migrated.p;
    r.jit = h->jit.p; r.accu = h->accu.p;
    r.tab_e = h->tab_e.p; r.tab_lg = h->tab_lg.p; r.tab_t = h->tab_t.p; r.tab_bad = h->tab_bad.p;
    r.cell_cnt = h->cell_cnt.p;
    r.rs_para = h->rs_para.p; r.CS = CS;
    r.sub_order = h->sub_order.p;
    r.res_order = h->res_order.p;
    r.lvl_ns = h->lvl_ns.p;
    r.pjit = h->pjit.p; r.paccu = h->paccu.p;
    r.prior = (!hier && !hyper) ? h->prior.p : nullptr;
    r.pp_bounds = (hier || hyper) ? h->pp_bounds.p : nullptr;
    r.phi_tab = hier ? h->phi_tab.p : nullptr;
    r.pth = h->pth.p; r.plp = h->plp.p; r.pll = h->pll.p;
    r.pth_s = h->pth_s.p; r.plp_s = h->plp_s.p; r.pll_s = h->pll_s.p;
    r.pref_src = h->pref_src.p; r.pref_next = h->pref_next.p;
    r.ppartner = h->ppartner.p; r.pneed = h->pneed.p; r.pptype = h->pptype.p;
    r.pnstep = h->pnstep.p; r.psub = h->psub.p; r.pmigrated = h->pmigrated.p;
    r.hprior = (hier || hyper) ? h->hprior.p : nullptr;
    r.hrows = hyper ? h->hrows.p : nullptr;
    r.n_row = hyper ? a.n_row : 0;
    r.smp_th = h->smp_th.p; r.smp_lp = h->smp_lp.p; r.smp_ll = h->smp_ll.p;
    r.psmp_th = h->psmp_th.p; r.psmp_lp = h->psmp_lp.p; r.psmp_ll = h->psmp_ll.p;
    r.stats = h->stats.p;
    r.status = h->status.p;
    r.ready = fused ? h->ready.p : nullptr;
    r.spec_cnt = fused ? h->spec_cnt.p : nullptr;
    r.ctl = fused ? h->ctl.p : nullptr;
    r.iter_end = (int32_t)n_iter;
    // migration steps evaluated ahead per resolve round: 4 measured 4% faster
    // than 8 and 2% faster than 3 on the 256-subject workload
    r.mig_round = h->tuning.mig_round > 0 ? h->tuning.mig_round : 4;
    if (const char *mr = std::getenv("GGDMC_MIG_ROUND")) r.mig_round = std::max(1, std::atoi(mr));
    r.lik_variant = h->tuning.lik_variant == 2 ? 1 : 0;
    if (const char *lv = std::getenv("GGDMC_LIK_VARIANT")) r.lik_variant = std::atoi(lv) == 2 ? 1 : 0;
    // GGDMC_SPEC_IDLE_LIMIT: polls before an idle CTA of the fused schedule
    // gives up waiting (default 2^21, about 2 s); the run then completes and
    // returns GGDMC_ERR_TIMEOUT
    r.spec_idle_limit = 1 << 21;
    if (const char *il = std::getenv("GGDMC_SPEC_IDLE_LIMIT")) r.spec_idle_limit = std::max(0, std::atoi(il));

    int64_t launches_per_iter = 0;
    // One DE iteration (src/de.cpp:201-242 / 272-383) as a launch sequence.
    auto one_iteration = [&]() -> cudaError_t {
        cudaError_t e;
        // Hierarchical and batched: the first subject pass's proposals and
        // their speculative evaluation read nothing the phi level writes
        // (only their priors do), so they run on a second stream beside it,
        // at low priority so the phi level's small kernels get SMs first;
        // k_sub_resolve scores the priors after the join.
        // Fused: k_sub_step of the previous iteration has already built
        // this iteration's proposals and evaluated part of them; the propose
        // kernel skips those levels and k_sub_spec_rest takes the items left.
        const bool fork = hier && S > 0 && Pphi > 0 && !plain;
        if (fork) {
            if ((e = cudaEventRecord(h->ev_fork, st))) return e;
            if ((e = cudaStreamWaitEvent(h->stream2, h->ev_fork, 0))) return e;
            if ((e = launch_sub_propose(r, 0, true, fused, h->stream2))) return e;
            if (fused) e = launch_sub_spec_rest(r, spec_group, h->stream2);
            else e = launch_sub_loglik(r, h->items.p, n_spec_items, spec_group, h->stream2);
            if (e) return e;
            if ((e = cudaEventRecord(h->ev_join, h->stream2))) return e;
            launches_per_iter += 2;
        }
        if (Pphi > 0) {
            const int npass = hier ? (c.is_hblocked ? c.nparameter : 1)
                                   : (c.is_pblocked ? c.nparameter : 1);
            for (int p = 0; p < npass; ++p) {
                if ((e = launch_phi_propose(r, p, st))) return e;
                if ((e = launch_phi_eval(r, st))) return e;
                if ((e = launch_phi_resolve(r, p, st))) return e;
                launches_per_iter += 3;
            }
            if (hier) {
                if ((e = launch_phi_tables(r, st))) return e;
                ++launches_per_iter;
                // the subject pass's level order (it matters when its levels
                // take more than one wave), beside the speculative evaluation
                if (fork && S > h->n_sm) {
                    if ((e = launch_level_order(r, fused, st))) return e;
                    ++launches_per_iter;
                }
            }
        }
        if (S > 0) {
            const int npass = hier ? (c.is_pblocked ? c.nparameter / 2 : 1)
                                   : (c.is_pblocked ? c.nparameter : 1);
            for (int p = 0; p < npass; ++p) {
                if (fork && p == 0) {
                    if ((e = cudaStreamWaitEvent(st, h->ev_join, 0))) return e;
                    if (fused) e = launch_sub_step(r, true, true, spec_group, st);
                    else e = launch_sub_resolve(r, 0, 0, S, true, st);
                    if (e) return e;
                    ++launches_per_iter;
                    continue;
                }
                if (fused) {
                    if ((e = launch_sub_propose(r, p, false, true, st))) return e;
                    if ((e = launch_sub_spec_rest(r, spec_group, st))) return e;
                    if ((e = launch_sub_step(r, false, false, spec_group, st))) return e;
                    launches_per_iter += 3;
                    continue;
                }
                if ((e = launch_sub_propose(r, p, false, false, st))) return e;
                ++launches_per_iter;
                if (plain) {
                    for (int l = 0; l < S; ++l) {
                        if ((e = launch_sub_loglik(r, h->items_plain.p + (size_t)l * CS, CS, 1, st))) return e;
                        if ((e = launch_sub_resolve(r, p, l, 1, false, st))) return e;
                        launches_per_iter += 2;
                    }
                } else {
                    if ((e = launch_sub_loglik(r, h->items.p, n_spec_items, spec_group, st))) return e;
                    if ((e = launch_sub_resolve(r, p, 0, S, false, st))) return e;
                    launches_per_iter += 2;
                }
            }
        }
        if ((e = launch_store(r, st))) return e;
        if ((e = launch_next_iter(r, st))) return e;
        launches_per_iter += 2;
        return cudaSuccess;
    };

    // slot 0 = start state, then iterations 1..n_iter
    CU(launch_store(r, st));
    CU(launch_next_iter(r, st));
    int64_t launches = 2;
    double sweep_ms = 0.0;
    int64_t copied = 0;   // sample slots already in the caller's buffers
    // cfg->flags bit 0: flush L2 (a memset larger than L2) between
    // iterations and time only the iterations' kernels, by event nodes.
    const bool flush = (c.flags & GGDMC_FLAG_L2_FLUSH) != 0;
    if (n_iter > 0) {
        const char *gs = std::getenv("GGDMC_GRAPH_ITERS");
        int64_t per_graph = h->tuning.graph_iters > 0 ? std::min(64, h->tuning.graph_iters) : 8;
        if (gs) per_graph = std::max(1, std::atoi(gs));
        per_graph = std::min<int64_t>(per_graph, n_iter);
        // built-in choice: a divisor of n_iter near 8 saves capturing a
        // second graph for the remainder
        if (!gs && h->tuning.graph_iters <= 0)
            for (int64_t dv = per_graph; dv >= std::max<int64_t>(4, per_graph / 2); --dv)
                if (n_iter % dv == 0) {
                    per_graph = dv;
                    break;
                }
        if (flush) CU(h->flushbuf.alloc(kFlushBytes));
        std::vector<cudaEvent_t> ev_a(per_graph + 1), ev_b(per_graph + 1);
        for (auto &e : ev_a) CU(cudaEventCreate(&e));
        for (auto &e : ev_b) CU(cudaEventCreate(&e));
        auto cleanup_events = [&]() {
            for (auto &e : ev_a) cudaEventDestroy(e);
            for (auto &e : ev_b) cudaEventDestroy(e);
        };
        // two graphs: per_graph iterations, replayed while at least that many
        // remain, and the remainder (n_iter % per_graph), so that every
        // iteration runs from a graph and its samples leave by the pipeline
        cudaGraph_t graph = nullptr, graph_tail = nullptr;
        cudaGraphExec_t exec = nullptr, exec_tail = nullptr;
        t_setup = ms_since(t_in);
        const auto t_cap = std::chrono::steady_clock::now();
        const int64_t rem = n_iter % per_graph;
        auto capture = [&](int64_t iters, cudaGraph_t &g, cudaGraphExec_t &x) -> ggdmc_status {
            CU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            cudaError_t ce = cudaSuccess;
            launches_per_iter = 0;
            for (int64_t i = 0; i < iters && ce == cudaSuccess; ++i) {
                // external event nodes: recorded (and timeable) on every replay
                if (flush) ce = cudaEventRecordWithFlags(ev_a[i], st, cudaEventRecordExternal);
                if (!ce) ce = one_iteration();
                if (flush && !ce) ce = cudaEventRecordWithFlags(ev_b[i], st, cudaEventRecordExternal);
                if (flush && !ce) ce = cudaMemsetAsync(h->flushbuf.p, (int)(i & 0xff), kFlushBytes, st);
            }
            cudaError_t ee = cudaStreamEndCapture(st, &g);
            if (ce || ee) return fail(GGDMC_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce ? ce : ee));
            cudaError_t ie = cudaGraphInstantiateWithFlags(&x, g, cudaGraphInstantiateFlagUseNodePriority);
            if (ie) return fail(GGDMC_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie));
            return GGDMC_OK;
        };
        auto destroy_graphs = [&]() {
            if (exec) cudaGraphExecDestroy(exec);
            if (graph) cudaGraphDestroy(graph);
            if (exec_tail) cudaGraphExecDestroy(exec_tail);
            if (graph_tail) cudaGraphDestroy(graph_tail);
        };
        ggdmc_status cs_ = rem ? capture(rem, graph_tail, exec_tail) : GGDMC_OK;
        if (!cs_) cs_ = capture(per_graph, graph, exec);
        if (cs_) {
            cleanup_events();
            destroy_graphs();
            return cs_;
        }
        const int64_t per_iter = launches_per_iter / per_graph;
        int64_t done = 0;
        ggdmc_status ws = GGDMC_OK;

        // Samples go to the caller while later sweeps run: after replay j,
        // one strided copy per array takes the slots it stored, for every
        // level, into page-locked stage j % 2 (second stream), and the host
        // moves chunk j - 1 into the caller's buffers while replay j runs.
        // Not with the L2-flush timing, which waits on every replay anyway.
        const bool want_subj = S > 0 && a.subj_out, want_phi = Pphi > 0 && a.phi_out;
        const bool pipe = !flush && (want_subj || want_phi);
        const size_t rth = (size_t)C * P, rph = (size_t)C * Pphi;   // doubles per slot
        auto slots_after = [&](int64_t iters) { return std::min<int64_t>(nmc, iters / c.thin + 1); };
        int64_t chunk_lo[2] = {0, 0}, chunk_hi[2] = {0, 0}, enq_hi = 0, rep = 0;
        cudaEvent_t ev_rep[2] = {}, ev_cp[2] = {};
        auto destroy_pipe = [&]() {
            for (int b = 0; b < 2; ++b) {
                if (ev_rep[b]) cudaEventDestroy(ev_rep[b]);
                if (ev_cp[b]) cudaEventDestroy(ev_cp[b]);
            }
        };
        if (pipe) {
            const int64_t ns_max = std::min<int64_t>(nmc, per_graph / c.thin + 2);
            size_t bytes = 0;
            if (want_subj) bytes += sizeof(double) * (size_t)S * ns_max * C * (P + 2);
            if (want_phi) bytes += sizeof(double) * (size_t)ns_max * C * (Pphi + 2);
            cudaError_t pe = cudaSuccess;
            for (int b = 0; b < 2 && !pe; ++b) {
                pe = h->stage[b].alloc(bytes);
                if (!pe) pe = cudaEventCreateWithFlags(&ev_rep[b], cudaEventDisableTiming);
                if (!pe) pe = cudaEventCreateWithFlags(&ev_cp[b], cudaEventDisableTiming);
            }
            if (pe) {
                destroy_pipe();
                cleanup_events();
                destroy_graphs();
                return fail(GGDMC_ERR_CUDA, std::string("sample staging: ") + cudaGetErrorString(pe));
            }
        }
        auto enqueue = [&](int b, int64_t lo, int64_t hi) -> cudaError_t {
            chunk_lo[b] = lo;
            chunk_hi[b] = hi;
            if (hi <= lo) return cudaSuccess;
            const size_t ns = (size_t)(hi - lo);
            cudaStream_t s2 = h->stream2;
            cudaError_t e = cudaStreamWaitEvent(s2, ev_rep[b], 0);
            char *dst = h->stage[b].p;
            const auto rows = [&](const double *src, size_t row, size_t n_row) -> cudaError_t {
                // n_row levels of ns slots each, source pitch nmc slots
                const size_t w = sizeof(double) * ns * row;
                cudaError_t ce = cudaMemcpy2DAsync(dst, w, src + (size_t)lo * row, sizeof(double) * nmc * row, w,
                                                   n_row, cudaMemcpyDeviceToHost, s2);
                dst += w * n_row;
                return ce;
            };
            if (want_subj) {
                if (!e) e = rows(h->smp_th.p, rth, S);
                if (!e) e = rows(h->smp_lp.p, C, S);
                if (!e) e = rows(h->smp_ll.p, C, S);
            }
            if (want_phi) {
                if (!e) e = rows(h->psmp_th.p, rph, 1);
                if (!e) e = rows(h->psmp_lp.p, C, 1);
                if (!e) e = rows(h->psmp_ll.p, C, 1);
            }
            if (!e) e = cudaEventRecord(ev_cp[b], s2);
            return e;
        };
        auto drain = [&](int b) -> ggdmc_status {
            const int64_t lo = chunk_lo[b], hi = chunk_hi[b];
            if (hi <= lo) return GGDMC_OK;
            ggdmc_status w = wait_event(ev_cp[b]);
            if (w) return w;
            const size_t ns = (size_t)(hi - lo);
            const char *src = h->stage[b].p;
            const auto put = [&](double *to, size_t row) {
                if (to) std::memcpy(to + (size_t)lo * row, src, sizeof(double) * ns * row);
                src += sizeof(double) * ns * row;
            };
            if (want_subj) {
                for (int l = 0; l < S; ++l) put(a.subj_out[l].theta, rth);
                for (int l = 0; l < S; ++l) put(a.subj_out[l].lp, C);
                for (int l = 0; l < S; ++l) put(a.subj_out[l].ll, C);
            }
            if (want_phi) {
                put(a.phi_out->theta, rph);
                put(a.phi_out->lp, C);
                put(a.phi_out->ll, C);
            }
            copied = hi;
            return GGDMC_OK;
        };

        t_capture = ms_since(t_cap);
        const auto t_rep = std::chrono::steady_clock::now();
        if (!flush) CU(cudaEventRecord(ev_a[per_graph], st));
        while (done < n_iter && !ws) {
            const bool full = done + per_graph <= n_iter;
            const int64_t iters = full ? per_graph : rem;
            cudaError_t e = cudaGraphLaunch(full ? exec : exec_tail, st);
            if (e) {
                ws = fail(GGDMC_ERR_CUDA, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
                break;
            }
            done += iters;
            if (pipe) {
                const int b = (int)(rep & 1);
                e = cudaEventRecord(ev_rep[b], st);
                const int64_t hi = slots_after(done);
                if (!e) e = enqueue(b, enq_hi, hi);
                if (e) {
                    ws = fail(GGDMC_ERR_CUDA, std::string("sample copy: ") + cudaGetErrorString(e));
                    break;
                }
                enq_hi = std::max(enq_hi, hi);
                if (rep >= 1) ws = drain(b ^ 1);
                ++rep;
                continue;
            }
            if (!flush) continue;
            // read this replay's event nodes before the next replay reuses them
            ws = wait_stream(st);
            if (ws) break;
            for (int64_t i = 0; i < iters && !ws; ++i) {
                float ms = 0.f;
                cudaError_t te = cudaEventElapsedTime(&ms, ev_a[i], ev_b[i]);
                if (te) ws = fail(GGDMC_ERR_CUDA, std::string("cudaEventElapsedTime: ") +
                                                      cudaGetErrorString(te));
                sweep_ms += ms;
            }
        }
        if (!flush && !ws) {
            CU(cudaEventRecord(ev_b[per_graph], st));
            ws = wait_stream(st);
            float ms = 0.f;
            if (!ws) cudaEventElapsedTime(&ms, ev_a[per_graph], ev_b[per_graph]);
            sweep_ms += ms;
        }
        if (pipe && rep >= 1 && !ws) ws = drain((int)((rep - 1) & 1));
        launches += n_iter * per_iter;
        t_run = ms_since(t_rep);
        destroy_graphs();
        cleanup_events();
        destroy_pipe();
        if (ws) return ws;
    }

    // ---- copy back: final state and samples
    if (n_iter == 0) t_setup = ms_since(t_in);
    const auto t_out = std::chrono::steady_clock::now();
    if (S > 0) {
        std::vector<double> buf((size_t)S * C * P), b1((size_t)S * C), b2((size_t)S * C);
        CU(cudaMemcpyAsync(buf.data(), h->th.p, sizeof(double) * buf.size(), cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(b1.data(), h->lp.p, sizeof(double) * b1.size(), cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(b2.data(), h->ll.p, sizeof(double) * b2.size(), cudaMemcpyDeviceToHost, st));
        { ggdmc_status ws_ = wait_stream(st); if (ws_) return ws_; }
        for (int l = 0; l < S; ++l) {
            const ggdmc_chain_state &cs = a.subj_state[l];
            std::memcpy(cs.theta, buf.data() + (size_t)l * C * P, sizeof(double) * C * P);
            std::memcpy(cs.lp, b1.data() + (size_t)l * C, sizeof(double) * C);
            std::memcpy(cs.ll, b2.data() + (size_t)l * C, sizeof(double) * C);
            if (a.subj_out && copied < nmc) {
                // the slots the pipelined copies have not delivered
                const ggdmc_samples &o = a.subj_out[l];
                const size_t k0 = (size_t)copied, nk = (size_t)(nmc - copied);
                if (o.theta)
                    CU(cudaMemcpyAsync(o.theta + k0 * C * P, h->smp_th.p + ((size_t)l * nmc + k0) * C * P,
                                       sizeof(double) * nk * C * P, cudaMemcpyDeviceToHost, st));
                if (o.lp)
                    CU(cudaMemcpyAsync(o.lp + k0 * C, h->smp_lp.p + ((size_t)l * nmc + k0) * C,
                                       sizeof(double) * nk * C, cudaMemcpyDeviceToHost, st));
                if (o.ll)
                    CU(cudaMemcpyAsync(o.ll + k0 * C, h->smp_ll.p + ((size_t)l * nmc + k0) * C,
                                       sizeof(double) * nk * C, cudaMemcpyDeviceToHost, st));
            }
        }
    }
    if (Pphi > 0) {
        const ggdmc_chain_state &ps = *a.phi_state;
        CU(cudaMemcpyAsync(ps.theta, h->pth.p, sizeof(double) * C * Pphi, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(ps.lp, h->plp.p, sizeof(double) * C, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(ps.ll, h->pll.p, sizeof(double) * C, cudaMemcpyDeviceToHost, st));
        if (a.phi_out && copied < nmc) {
            const ggdmc_samples &o = *a.phi_out;
            const size_t k0 = (size_t)copied, nk = (size_t)(nmc - copied);
            if (o.theta)
                CU(cudaMemcpyAsync(o.theta + k0 * C * Pphi, h->psmp_th.p + k0 * C * Pphi,
                                   sizeof(double) * nk * C * Pphi, cudaMemcpyDeviceToHost, st));
            if (o.lp)
                CU(cudaMemcpyAsync(o.lp + k0 * C, h->psmp_lp.p + k0 * C, sizeof(double) * nk * C,
                                   cudaMemcpyDeviceToHost, st));
            if (o.ll)
                CU(cudaMemcpyAsync(o.ll + k0 * C, h->psmp_ll.p + k0 * C, sizeof(double) * nk * C,
                                   cudaMemcpyDeviceToHost, st));
        }
    }
    unsigned long long hs[ST_N];
    int32_t dev_status = 0;
    CU(cudaMemcpyAsync(hs, h->stats.p, sizeof hs, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&dev_status, h->status.p, sizeof dev_status, cudaMemcpyDeviceToHost, st));
    if ((s = wait_stream(st))) return s;
    if (dev_status)
        return fail(GGDMC_ERR_TIMEOUT, "a device-side wait gave up (code " + std::to_string(dev_status) + ")");
    h->last_nmc = nmc; h->last_C = C; h->last_P = P; h->last_Pphi = Pphi; h->last_S = S;
    if (a.stats) {
        a.stats->proposals = (int64_t)hs[ST_PROPOSALS];
        a.stats->accepts = (int64_t)hs[ST_ACCEPTS];
        a.stats->migrations = (int64_t)hs[ST_MIGRATIONS];
        a.stats->reevaluations = (int64_t)hs[ST_REEVALS];
        a.stats->kernel_launches = launches;
        a.stats->trial_evals = (int64_t)hs[ST_TRIALS];
        a.stats->resolve_rounds = (int64_t)hs[ST_ROUNDS];
        a.stats->variants = (int64_t)hs[ST_VARIANTS];
        a.stats->fallbacks = (int64_t)hs[ST_FALLBACKS];
        a.stats->iterations = n_iter;
        a.stats->sweep_ms = sweep_ms;
        a.stats->setup_ms = t_setup;
        a.stats->capture_ms = t_capture;
        a.stats->run_ms = t_run;
        a.stats->copyout_ms = ms_since(t_out);
    }
    return GGDMC_OK;
}

void release_streams(ggdmc_handle *h)
{
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->stream2) cudaStreamSynchronize(h->stream2);
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->stream2) cudaStreamDestroy(h->stream2);
    if (h->stream) cudaStreamDestroy(h->stream);
}

ggdmc_status make_handle(const ggdmc_model *model, const ggdmc_data *data, ggdmc_handle **out)
{
    if (!out) return fail(GGDMC_ERR_ARG, "out is NULL");
    *out = nullptr;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev < 1)
        return fail(GGDMC_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    auto *h = new ggdmc_handle();
    cudaGetDevice(&h->device);
    cudaDeviceGetAttribute(&h->n_sm, cudaDevAttrMultiProcessorCount, h->device);
    if (h->n_sm < 1) h->n_sm = 1;
    int prio_low = 0, prio_high = 0;
    e = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high);
    if (!e) e = cudaStreamCreateWithPriority(&h->stream, cudaStreamNonBlocking, prio_high);
    if (!e) e = cudaStreamCreateWithPriority(&h->stream2, cudaStreamNonBlocking, prio_low);
    if (!e) e = cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming);
    if (!e) e = cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming);
    ggdmc_status s = e ? fail(GGDMC_ERR_CUDA, std::string("stream / event create: ") + cudaGetErrorString(e))
                       : GGDMC_OK;
    if (!s && model) s = build_design(h, model);
    if (!s) s = upload_data(h, data);
    if (s) {
        release_streams(h);
        delete h;
        return s;
    }
    *out = h;
    return GGDMC_OK;
}

// Rejection draws of one level set (S levels x C chains of P parameters) until
// every pair has a finite prior and likelihood; score() fills d_ll from
// d_theta.  On return the host arrays hold theta, lp and ll.
template <class Score>
static ggdmc_status init_level(ggdmc_handle *h, const ggdmc_prior *prior, int S, int C, int P, int level0,
                               int max_attempts, uint64_t seed, DevBuf<double> &d_theta, Score score,
                               std::vector<double> &th, std::vector<double> &lp, std::vector<double> &ll)
{
    cudaStream_t st = h->stream;
    std::vector<double> rows;
    ggdmc_status s = prior_rows(prior, rows);
    if (s) return s;
    const size_t n = (size_t)S * C;
    DevBuf<double> d_rows, d_lp, d_ll;
    DevBuf<int32_t> d_att;
    DevBuf<uint8_t> d_done;
    CU(d_rows.upload(rows.data(), rows.size(), st));
    CU(d_theta.alloc(n * P));
    CU(d_lp.alloc(n));
    CU(d_ll.alloc(n));
    std::vector<int32_t> att(n, 0);
    std::vector<uint8_t> done(n, 0);
    lp.assign(n, 0.0);
    ll.assign(n, 0.0);
    size_t left = n;
    for (int a = 0; a < max_attempts && left; ++a) {
        CU(d_att.upload(att.data(), n, st));
        CU(d_done.upload(done.data(), n, st));
        CU(launch_init_draw(d_rows.p, P, C, level0, S, d_att.p, d_done.p, seed, d_theta.p, st));
        CU(launch_logprior(d_rows.p, P, d_theta.p, (int)n, d_lp.p, st));
        CU(score(d_theta.p, d_ll.p));
        std::vector<double> lp_a(n), ll_a(n);
        CU(cudaMemcpyAsync(lp_a.data(), d_lp.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(ll_a.data(), d_ll.p, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
        if ((s = wait_stream(st))) return s;
        for (size_t i = 0; i < n; ++i) {
            if (done[i]) continue;
            if (std::isfinite(lp_a[i]) && std::isfinite(ll_a[i])) {
                done[i] = 1;
                lp[i] = lp_a[i];
                ll[i] = ll_a[i];
                --left;
            } else {
                ++att[i];
            }
        }
    }
    if (left)
        return fail(GGDMC_ERR_NUMERIC, std::to_string(left) + " chain(s) found no start with a finite prior and "
                                       "likelihood in " + std::to_string(max_attempts) + " attempts");
    th.resize(n * P);
    CU(cudaMemcpyAsync(th.data(), d_theta.p, sizeof(double) * n * P, cudaMemcpyDeviceToHost, st));
    return wait_stream(st);
}

}  // namespace

// ================================================================== C ABI
extern "C" {

const char *ggdmc_last_error(void) { return g_err.c_str(); }

const char *ggdmc_version(void) { return "ggdmc_gb300 0.1 (sm_103a)"; }

ggdmc_status ggdmc_draw_layout(const ggdmc_de_config *cfg, int32_t n_level, int32_t hierarchical,
                               int64_t *n_iter, int64_t *n_pass, int64_t *n_slot, int64_t *total)
{
    ggdmc_status s = check_cfg(cfg);
    if (s) return s;
    int64_t np = 1;
    if (hierarchical)
        np = std::max<int64_t>(cfg->is_hblocked ? cfg->nparameter : 1,
                               cfg->is_pblocked ? cfg->nparameter / 2 : 1);
    else if (cfg->is_pblocked)
        np = cfg->nparameter;
    const int64_t ni = (int64_t)(cfg->nmc - 1) * cfg->thin;
    const int64_t ns = GGDMC_DRAW_SLOTS(cfg->nchain, cfg->nparameter);
    if (n_iter) *n_iter = ni;
    if (n_pass) *n_pass = np;
    if (n_slot) *n_slot = ns;
    if (total) *total = ni * n_level * np * ns;
    return GGDMC_OK;
}

ggdmc_status ggdmc_create(const ggdmc_model *model, const ggdmc_data *data, ggdmc_handle **out)
{
    if (!model) return fail(GGDMC_ERR_ARG, "model is NULL");
    return make_handle(model, data, out);
}

ggdmc_status ggdmc_destroy(ggdmc_handle *h)
{
    if (!h) return GGDMC_OK;
    release_streams(h);
    delete h;
    return GGDMC_OK;
}

// A one-shot call: a handle for the call's design and trials, the run, the
// release; the handle's creation counts into setup_ms and its release into
// copyout_ms.
static ggdmc_status run_oneshot(const ggdmc_model *model, const ggdmc_data *data, const RunArgs &a)
{
    const auto t0 = std::chrono::steady_clock::now();
    ggdmc_handle *h = nullptr;
    ggdmc_status s = make_handle(model, data, &h);
    if (s) return s;
    const double t_make = ms_since(t0);
    // settings the autotuner found for this shape earlier in the process
    if (model && data && a.cfg) {
        char key[512];
        ggdmc_tuning t{};
        if (!ggdmc_tune_key(model, data, a.cfg->nchain, a.kind == RK_HIER, key, sizeof key) &&
            !ggdmc_tune_lookup(key, nullptr, &t))
            h->tuning = t;
        g_err.clear();
    }
    s = run_impl(h, a);
    const std::string keep = g_err;
    const auto t1 = std::chrono::steady_clock::now();
    ggdmc_destroy(h);
    g_err = keep;
    if (a.stats && !s) {
        a.stats->setup_ms += t_make;
        a.stats->copyout_ms += ms_since(t1);
    }
    return s;
}

ggdmc_status ggdmc_handle_run(ggdmc_handle *h, const ggdmc_de_config *cfg, const ggdmc_prior *p_prior,
                              const ggdmc_prior *h_prior, ggdmc_chain_state *phi_state,
                              ggdmc_chain_state *subj_state, const double *draws,
                              ggdmc_samples *phi_out, ggdmc_samples *subj_out, ggdmc_run_stats *stats)
{
    if (!h) return fail(GGDMC_ERR_ARG, "handle is NULL");
    RunArgs a{phi_state ? RK_HIER : RK_SUBJECTS, cfg, p_prior, h_prior, phi_state, subj_state,
              draws, phi_out, subj_out, stats, nullptr, 0};
    return run_impl(h, a);
}

ggdmc_status ggdmc_run_subjects(const ggdmc_de_config *cfg, const ggdmc_model *model,
                                const ggdmc_data *data, const ggdmc_prior *p_prior,
                                ggdmc_chain_state *state, const double *draws, ggdmc_samples *out,
                                ggdmc_run_stats *stats)
{
    RunArgs a{RK_SUBJECTS, cfg, p_prior, nullptr, nullptr, state, draws, nullptr, out, stats,
              nullptr, 0};
    return run_oneshot(model, data, a);
}

ggdmc_status ggdmc_run_subject(const ggdmc_de_config *cfg, const ggdmc_model *model,
                               const ggdmc_data *data, const ggdmc_prior *p_prior,
                               ggdmc_chain_state *state, const double *draws, ggdmc_samples *out,
                               ggdmc_run_stats *stats)
{
    if (!data || data->n_subject != 1)
        return fail(GGDMC_ERR_ARG, "run_subject takes exactly one subject");
    return ggdmc_run_subjects(cfg, model, data, p_prior, state, draws, out, stats);
}

ggdmc_status ggdmc_run(const ggdmc_de_config *cfg, const ggdmc_model *model, const ggdmc_data *data,
                       const ggdmc_prior *p_prior, const ggdmc_prior *h_prior,
                       ggdmc_chain_state *phi_state, ggdmc_chain_state *subj_state,
                       const double *draws, ggdmc_samples *phi_out, ggdmc_samples *subj_out,
                       ggdmc_run_stats *stats)
{
    RunArgs a{RK_HIER, cfg, p_prior, h_prior, phi_state, subj_state, draws, phi_out, subj_out,
              stats, nullptr, 0};
    return run_oneshot(model, data, a);
}

ggdmc_status ggdmc_run_hyper(const ggdmc_de_config *cfg, const double *hyper_data, int32_t n_row,
                             const ggdmc_prior *p_prior, const ggdmc_prior *h_prior,
                             ggdmc_chain_state *state, const double *draws, ggdmc_samples *out,
                             ggdmc_run_stats *stats)
{
    RunArgs a{RK_HYPER, cfg, p_prior, h_prior, state, nullptr, draws, out, nullptr, stats,
              hyper_data, n_row};
    return run_oneshot(nullptr, nullptr, a);
}

static RunDev loglik_desc(ggdmc_handle *h, int prec)
{
    RunDev r{};
    r.P = h->n_par;
    r.S = h->S;
    r.prec = (prec == GGDMC_MIXED || prec == GGDMC_MIXED_SUMS) ? PREC_MIXED : PREC_FP64;
    r.m = h->dev_model();
    r.offs = h->offs.p; r.rt64 = h->rt64.p; r.rt32 = h->rt32.p; r.cell = h->cell.p;
    r.cell_cnt = h->cell_cnt.p;
    return r;
}

// The batch likelihood on device buffers; MIXED sums near zero are then
// recomputed in FP64 (launch_refine) so each sum is within 1e-6 relative.
static ggdmc_status loglik_launch(ggdmc_handle *h, const double *d_theta, int n_theta, int precision,
                                  double *d_out, cudaStream_t st)
{
    RunDev r = loglik_desc(h, precision);
    BatchTables bt{nullptr, nullptr, nullptr, nullptr};
    if (r.prec == PREC_MIXED && h->model_type != GGDMC_MODEL_DDM) {
        const size_t nq = (size_t)h->S * n_theta;
        CU(h->bt_e.alloc(nq * h->n_ent));
        CU(h->bt_lg.alloc(nq * h->n_ent));
        CU(h->bt_t.alloc(nq * std::max(h->n_t0, 1)));
        CU(h->bt_bad.alloc(nq));
        bt = BatchTables{h->bt_e.p, h->bt_lg.p, h->bt_t.p, h->bt_bad.p};
    }
    CU(launch_loglik_batch(r, d_theta, n_theta, d_out, st, &bt));
    if (precision != GGDMC_MIXED) return GGDMC_OK;
    const size_t cap = refine_capacity(h->h_offs.data(), h->S, n_theta);
    CU(h->ref_count.alloc(1));
    CU(h->ref_base.alloc((size_t)h->S * n_theta));
    CU(h->ref_item.alloc(std::max<size_t>(cap, 1)));
    CU(h->ref_partial.alloc(std::max<size_t>(cap, 1)));
    CU(launch_refine(r, d_theta, n_theta, d_out, h->ref_count.p, h->ref_base.p, h->ref_item.p, h->ref_partial.p,
                     4 * h->n_sm, st));
    return GGDMC_OK;
}

ggdmc_status ggdmc_loglik_device(ggdmc_handle *h, const double *d_theta, int32_t n_theta,
                                 int32_t precision, double *d_out, void *stream)
{
    if (!h || !d_theta || !d_out || n_theta < 1) return fail(GGDMC_ERR_ARG, "bad loglik arguments");
    if (h->S < 1) return fail(GGDMC_ERR_ARG, "handle has no subjects");
    return loglik_launch(h, d_theta, n_theta, precision, d_out, (cudaStream_t)stream);
}

ggdmc_status ggdmc_loglik(ggdmc_handle *h, const double *theta, int32_t n_theta, int32_t precision,
                          double *out)
{
    if (!h || !theta || !out || n_theta < 1) return fail(GGDMC_ERR_ARG, "bad loglik arguments");
    if (h->S < 1) return fail(GGDMC_ERR_ARG, "handle has no subjects");
    const size_t nt = (size_t)h->S * n_theta;
    CU(h->io_a.upload(theta, nt * h->n_par, h->stream));
    CU(h->io_b.alloc(nt));
    ggdmc_status s = loglik_launch(h, h->io_a.p, n_theta, precision, h->io_b.p, h->stream);
    if (s) return s;
    CU(cudaMemcpyAsync(out, h->io_b.p, sizeof(double) * nt, cudaMemcpyDeviceToHost, h->stream));
    return wait_stream(h->stream);
}

ggdmc_status ggdmc_initialise(ggdmc_handle *h, const ggdmc_prior *p_prior, const ggdmc_prior *h_prior,
                              int32_t nchain, int32_t max_attempts, uint64_t seed, int32_t precision,
                              ggdmc_chain_state *subj_state, ggdmc_chain_state *phi_state)
{
    if (!h || !p_prior || !subj_state || nchain < 1 || max_attempts < 1)
        return fail(GGDMC_ERR_ARG, "bad initialise arguments");
    if (h->S < 1) return fail(GGDMC_ERR_ARG, "handle has no subjects");
    if (p_prior->n_par != h->n_par) return fail(GGDMC_ERR_ARG, "p_prior must have one row per parameter");
    if (h_prior && (!phi_state || h_prior->n_par != 2 * h->n_par))
        return fail(GGDMC_ERR_ARG, "h_prior needs 2 x n_par rows and a phi_state");
    const int S = h->S, C = nchain, P = h->n_par;
    const RunDev lr = loglik_desc(h, precision);
    DevBuf<double> d_th;
    std::vector<double> th, lp, ll;
    ggdmc_status s = init_level(h, p_prior, S, C, P, 1, max_attempts, seed, d_th,
                                [&](const double *t, double *o) { return launch_loglik_batch(lr, t, C, o, h->stream); },
                                th, lp, ll);
    if (s) return s;
    for (int l = 0; l < S; ++l) {
        const ggdmc_chain_state &cs = subj_state[l];
        if (!cs.theta || !cs.lp || !cs.ll) return fail(GGDMC_ERR_ARG, "subject state incomplete");
        std::memcpy(cs.theta, th.data() + (size_t)l * C * P, sizeof(double) * C * P);
        std::memcpy(cs.lp, lp.data() + (size_t)l * C, sizeof(double) * C);
        std::memcpy(cs.ll, ll.data() + (size_t)l * C, sizeof(double) * C);
    }
    if (!h_prior) return GGDMC_OK;
    // phi: hyper log-likelihood against the subjects' chains c (src/de.cpp:245-270)
    if (2 * P > kMaxTheta) return fail(GGDMC_ERR_ARG, "too many parameters");
    std::vector<double> bounds(2 * (size_t)P);
    for (int j = 0; j < P; ++j) {
        bounds[2 * j] = p_prior->table[6 * j + 2];
        bounds[2 * j + 1] = p_prior->table[6 * j + 3];
    }
    DevBuf<double> d_b, d_phi;
    CU(d_b.upload(bounds.data(), bounds.size(), h->stream));
    RunDev hr{};
    hr.C = C; hr.P = P; hr.Pphi = 2 * P; hr.S = S;
    hr.th = d_th.p; hr.pp_bounds = d_b.p;
    hr.prec = (precision == GGDMC_MIXED) ? PREC_MIXED : PREC_FP64;
    std::vector<double> pth, plp, pll;
    s = init_level(h, h_prior, 1, C, 2 * P, 0, max_attempts, seed, d_phi,
                   [&](const double *t, double *o) { return launch_loghlike(hr, t, o, h->stream); }, pth, plp, pll);
    if (s) return s;
    if (!phi_state->theta || !phi_state->lp || !phi_state->ll) return fail(GGDMC_ERR_ARG, "phi state incomplete");
    std::memcpy(phi_state->theta, pth.data(), sizeof(double) * C * 2 * P);
    std::memcpy(phi_state->lp, plp.data(), sizeof(double) * C);
    std::memcpy(phi_state->ll, pll.data(), sizeof(double) * C);
    return GGDMC_OK;
}

ggdmc_status ggdmc_handle_summary(ggdmc_handle *h, int32_t start, double *mean, double *sd, double *psrf,
                                  double *phi_mean, double *phi_sd, double *phi_psrf)
{
    if (!h) return fail(GGDMC_ERR_ARG, "handle is NULL");
    if (h->last_nmc < 1) return fail(GGDMC_ERR_ARG, "no run has stored samples on this handle");
    const int nmc = h->last_nmc, C = h->last_C;
    if (start < 0 || nmc - start < 2 || C < 2)
        return fail(GGDMC_ERR_ARG, "summary needs two or more iterations after start and two or more chains");
    cudaStream_t st = h->stream;
    auto level = [&](const double *smp, int L, int P, double *m, double *s, double *r) -> ggdmc_status {
        if (L < 1 || P < 1) return GGDMC_OK;
        if (!m || !s || !r) return fail(GGDMC_ERR_ARG, "summary output is NULL");
        DevBuf<double> cs, dm, dsd, dr;
        CU(cs.alloc((size_t)L * C * P * 2));
        CU(dm.alloc((size_t)L * P));
        CU(dsd.alloc((size_t)L * P));
        CU(dr.alloc((size_t)L * P));
        CU(launch_summary(smp, L, nmc, C, P, start, cs.p, dm.p, dsd.p, dr.p, st));
        CU(cudaMemcpyAsync(m, dm.p, sizeof(double) * L * P, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(s, dsd.p, sizeof(double) * L * P, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(r, dr.p, sizeof(double) * L * P, cudaMemcpyDeviceToHost, st));
        return wait_stream(st);
    };
    ggdmc_status s = level(h->smp_th.p, h->last_S, h->last_P, mean, sd, psrf);
    if (s) return s;
    if (h->last_Pphi > 0 && phi_mean)
        s = level(h->psmp_th.p, 1, h->last_Pphi, phi_mean, phi_sd, phi_psrf);
    return s;
}

ggdmc_status ggdmc_handle_diagnostics(ggdmc_handle *h, int32_t start, int32_t end, const double *probs,
                                      int32_t n_prob, double conf, int32_t psrf_form, ggdmc_diag *subj,
                                      ggdmc_diag *phi)
{
    if (!h) return fail(GGDMC_ERR_ARG, "handle is NULL");
    if (h->last_nmc < 1) return fail(GGDMC_ERR_ARG, "no run has stored samples on this handle");
    const int nmc = h->last_nmc, C = h->last_C;
    if (end <= 0) end = nmc;
    if (start < 0 || end > nmc || end - start < 2)
        return fail(GGDMC_ERR_ARG, "diagnostics need 0 <= start, end <= nmc and two or more iterations");
    const int n = end - start;
    if (diag_kmax(n) > kDiagMaxLag) return fail(GGDMC_ERR_ARG, "diagnostics take at most 2.5e6 iterations");
    if (n_prob == 1) return fail(GGDMC_ERR_ARG, "prob must be more than one element");
    if (n_prob < 0 || n_prob > kDiagMaxProb || (n_prob > 0 && !probs))
        return fail(GGDMC_ERR_ARG, "n_prob must be 0 or 2..16 with probs given");
    for (int i = 0; i < n_prob; ++i)
        if (!(probs[i] >= 0.0 && probs[i] <= 1.0)) return fail(GGDMC_ERR_ARG, "probs must lie in [0, 1]");
    if (psrf_form != GGDMC_PSRF_REFERENCE && psrf_form != GGDMC_PSRF_CODA)
        return fail(GGDMC_ERR_ARG, "psrf_form must be GGDMC_PSRF_REFERENCE or GGDMC_PSRF_CODA");
    cudaStream_t st = h->stream;
    DevBuf<double> dprobs;
    if (n_prob > 0) {
        CU(dprobs.alloc(n_prob));
        CU(cudaMemcpyAsync(dprobs.p, probs, sizeof(double) * n_prob, cudaMemcpyHostToDevice, st));
    }
    auto level = [&](const double *smp, int L, int P, ggdmc_diag *o) -> ggdmc_status {
        if (!o || L < 1 || P < 1) return GGDMC_OK;
        if (o->psrf && C < 3) return fail(GGDMC_ERR_ARG, "Minimum three chains needed");
        if (o->psrf && !(conf > 0.0 && conf < 1.0)) return fail(GGDMC_ERR_ARG, "conf must lie in (0, 1)");
        const bool wform = o->psrf && psrf_form == GGDMC_PSRF_REFERENCE;
        if (wform && P > kDiagMaxPsrfPar)
            return fail(GGDMC_ERR_ARG, "the reference PSRF form takes at most 64 parameters a level");
        const size_t LP = (size_t)L * P;
        DevBuf<double> cstat, wcov, out;
        CU(cstat.alloc(LP * C * 3));
        if (wform) CU(wcov.alloc(LP * C * P));
        // outputs side by side: mean, sd, naive, ts [LP] each, quantiles [LP][n_prob], psrf [LP][2]
        const size_t oq = 4 * LP, opsrf = oq + LP * n_prob, ntot = opsrf + 2 * LP;
        CU(out.alloc(ntot));
        double *q = out.p;
        CU(launch_diagnostics(smp, L, nmc, C, P, start, n, dprobs.p, o->quantiles ? n_prob : 0, conf, psrf_form,
                              cstat.p, wcov.p, q, q + LP, q + 2 * LP, q + 3 * LP,
                              (o->quantiles && n_prob > 0) ? q + oq : nullptr, o->psrf ? q + opsrf : nullptr, st));
        std::vector<double> host(ntot);
        CU(cudaMemcpyAsync(host.data(), out.p, sizeof(double) * ntot, cudaMemcpyDeviceToHost, st));
        ggdmc_status ws = wait_stream(st);
        if (ws) return ws;
        auto put = [&](double *dst, size_t off, size_t cnt) {
            if (dst) std::memcpy(dst, host.data() + off, sizeof(double) * cnt);
        };
        put(o->mean, 0, LP);
        put(o->sd, LP, LP);
        put(o->naive_se, 2 * LP, LP);
        put(o->ts_se, 3 * LP, LP);
        if (n_prob > 0) put(o->quantiles, oq, LP * n_prob);
        put(o->psrf, opsrf, 2 * LP);
        return GGDMC_OK;
    };
    ggdmc_status s = level(h->smp_th.p, h->last_S, h->last_P, subj);
    if (s) return s;
    if (h->last_Pphi > 0) s = level(h->psmp_th.p, 1, h->last_Pphi, phi);
    return s;
}

ggdmc_status ggdmc_trial_logdens(ggdmc_handle *h, const double *theta, int32_t precision, double *out)
{
    if (!h || !theta || !out) return fail(GGDMC_ERR_ARG, "bad trial_logdens arguments");
    if (h->S < 1) return fail(GGDMC_ERR_ARG, "handle has no subjects");
    const size_t N = (size_t)h->h_offs[h->S];
    CU(h->io_a.upload(theta, (size_t)h->S * h->n_par, h->stream));
    CU(h->io_b.alloc(std::max<size_t>(N, 1)));
    RunDev r = loglik_desc(h, precision);
    CU(launch_trial_logdens(r, h->io_a.p, h->io_b.p, h->stream));
    std::vector<double> dev(N);
    if (N) CU(cudaMemcpyAsync(dev.data(), h->io_b.p, sizeof(double) * N, cudaMemcpyDeviceToHost, h->stream));
    ggdmc_status ws = wait_stream(h->stream);
    if (ws) return ws;
    for (size_t j = 0; j < N; ++j) out[h->perm[j]] = dev[j];   // back to the data's trial order
    return GGDMC_OK;
}

ggdmc_status ggdmc_logprior(const ggdmc_prior *prior, const double *theta, int32_t n, double *out)
{
    if (!theta || !out || n < 1) return fail(GGDMC_ERR_ARG, "bad logprior arguments");
    std::vector<double> rows;
    ggdmc_status s = prior_rows(prior, rows);
    if (s) return s;
    const int P = prior->n_par;
    double *d_rows = nullptr, *d_th = nullptr, *d_out = nullptr;
    cudaError_t e = cudaMalloc(&d_rows, sizeof(double) * rows.size());
    if (!e) e = cudaMalloc(&d_th, sizeof(double) * (size_t)n * P);
    if (!e) e = cudaMalloc(&d_out, sizeof(double) * n);
    if (!e) e = cudaMemcpy(d_rows, rows.data(), sizeof(double) * rows.size(), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(d_th, theta, sizeof(double) * (size_t)n * P, cudaMemcpyHostToDevice);
    if (!e) e = launch_logprior(d_rows, P, d_th, n, d_out, nullptr);
    if (!e) e = cudaMemcpy(out, d_out, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(d_rows);
    cudaFree(d_th);
    cudaFree(d_out);
    if (e) return fail(GGDMC_ERR_CUDA, std::string("logprior: ") + cudaGetErrorString(e));
    return GGDMC_OK;
}

ggdmc_status ggdmc_logprior_noalloc(const ggdmc_prior *prior, const double *theta, int32_t n, double *out)
{
    if (!theta || !out || n < 1) return fail(GGDMC_ERR_ARG, "bad logprior arguments");
    std::vector<double> rows;
    ggdmc_status s = prior_rows(prior, rows);
    if (s) return s;
    const int P = prior->n_par;
    const size_t n_rows = rows.size(), n_th = (size_t)n * P;
    const size_t need = round256(n_rows) + round256(n_th) + round256((size_t)n);
    if (need > kScratchDoubles)
        return fail(GGDMC_ERR_ARG, "logprior_noalloc: " + std::to_string(n) + " vectors of " +
                                       std::to_string(P) + " parameters need " + std::to_string(need * 8) +
                                       " bytes of scratch; the limit is " +
                                       std::to_string(kScratchDoubles * 8) + " bytes");
    double *base = nullptr;
    s = scratch_base(&base);
    if (s) return s;
    double *d_rows = base, *d_th = d_rows + round256(n_rows), *d_out = d_th + round256(n_th);
    CU(cudaMemcpy(d_rows, rows.data(), sizeof(double) * n_rows, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(d_th, theta, sizeof(double) * n_th, cudaMemcpyHostToDevice));
    CU(launch_logprior(d_rows, P, d_th, n, d_out, nullptr));
    CU(cudaMemcpy(out, d_out, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return GGDMC_OK;
}

ggdmc_status ggdmc_loghlike(const ggdmc_prior *p_prior, const double *phi, const double *subj_theta,
                            int32_t n_subject, int32_t n, double *out)
{
    if (!p_prior || !phi || !subj_theta || !out || n < 1 || n_subject < 1)
        return fail(GGDMC_ERR_ARG, "bad loghlike arguments");
    const int P = p_prior->n_par;
    if (2 * P > kMaxTheta) return fail(GGDMC_ERR_ARG, "too many parameters");
    std::vector<double> bounds(2 * (size_t)P);
    for (int j = 0; j < P; ++j) {
        bounds[2 * j] = p_prior->table[6 * j + 2];
        bounds[2 * j + 1] = p_prior->table[6 * j + 3];
    }
    double *d_b = nullptr, *d_phi = nullptr, *d_th = nullptr, *d_out = nullptr;
    cudaError_t e = cudaMalloc(&d_b, sizeof(double) * bounds.size());
    if (!e) e = cudaMalloc(&d_phi, sizeof(double) * (size_t)n * 2 * P);
    if (!e) e = cudaMalloc(&d_th, sizeof(double) * (size_t)n_subject * n * P);
    if (!e) e = cudaMalloc(&d_out, sizeof(double) * n);
    if (!e) e = cudaMemcpy(d_b, bounds.data(), sizeof(double) * bounds.size(), cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(d_phi, phi, sizeof(double) * (size_t)n * 2 * P, cudaMemcpyHostToDevice);
    if (!e) e = cudaMemcpy(d_th, subj_theta, sizeof(double) * (size_t)n_subject * n * P,
                           cudaMemcpyHostToDevice);
    if (!e) {
        RunDev r{};
        r.C = n; r.P = P; r.Pphi = 2 * P; r.S = n_subject;
        r.th = d_th; r.pp_bounds = d_b;
        e = launch_loghlike(r, d_phi, d_out, nullptr);
    }
    if (!e) e = cudaMemcpy(out, d_out, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(d_b);
    cudaFree(d_phi);
    cudaFree(d_th);
    cudaFree(d_out);
    if (e) return fail(GGDMC_ERR_CUDA, std::string("loghlike: ") + cudaGetErrorString(e));
    return GGDMC_OK;
}

// ------------------------------------------------------------ tuning
namespace {

std::mutex g_tune_mu;
std::map<std::string, ggdmc_tuning> g_tune_cache;   // this process's autotuner cache

int pow2_floor(int64_t x)
{
    int k = 0;
    while (x > 1) {
        x >>= 1;
        ++k;
    }
    return k;
}

}  // namespace

ggdmc_status ggdmc_tune_key(const ggdmc_model *model, const ggdmc_data *data, int32_t nchain, int32_t hierarchical,
                            char *key, int32_t key_len)
{
    if (!model || !data || !key || key_len < 1 || !data->offsets || data->n_subject < 0)
        return fail(GGDMC_ERR_ARG, "bad tune_key arguments");
    // trial counts by power of two; each bin's subject count by power of two
    std::map<int, int64_t> bins;
    for (int s = 0; s < data->n_subject; ++s) ++bins[pow2_floor(data->offsets[s + 1] - data->offsets[s])];
    std::string k = (model->model_type == GGDMC_MODEL_DDM ? "ddm" : "lba") + std::to_string(model->n_acc) + ".p" +
                    std::to_string(model->n_par) + ".c" + std::to_string(nchain) + (hierarchical ? ".h" : ".f") +
                    ".s" + std::to_string(pow2_floor(std::max(data->n_subject, 1)));
    for (const auto &b : bins) k += "." + std::to_string(b.first) + "x" + std::to_string(pow2_floor(b.second));
    if ((int32_t)k.size() + 1 > key_len) return fail(GGDMC_ERR_ARG, "key buffer too small");
    std::memcpy(key, k.c_str(), k.size() + 1);
    return GGDMC_OK;
}

ggdmc_status ggdmc_tune_lookup(const char *key, const char *cache_path, ggdmc_tuning *out)
{
    if (!key || !out) return fail(GGDMC_ERR_ARG, "bad tune_lookup arguments");
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            *out = it->second;
            return GGDMC_OK;
        }
    }
    if (cache_path) {
        if (FILE *f = std::fopen(cache_path, "r")) {
            char kb[512];
            ggdmc_tuning t{}, found{};
            bool hit = false;
            while (std::fscanf(f, "%511s %d %d %d %d %lf", kb, &t.spec_group, &t.graph_iters, &t.mig_round,
                               &t.lik_variant, &t.sweep_ms) == 6)
                if (std::strcmp(kb, key) == 0) {
                    found = t;
                    hit = true;
                }
            std::fclose(f);
            if (hit) {
                std::lock_guard<std::mutex> lk(g_tune_mu);
                g_tune_cache[key] = found;
                *out = found;
                return GGDMC_OK;
            }
        }
    }
    return fail(GGDMC_ERR_ARG, "no tuning cached for this key");
}

ggdmc_status ggdmc_tune_store(const char *key, const char *cache_path, const ggdmc_tuning *t)
{
    if (!key || !t || !*key || std::strchr(key, ' ') || std::strchr(key, '\n'))
        return fail(GGDMC_ERR_ARG, "bad tune_store arguments");
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = *t;
    }
    if (cache_path) {
        FILE *f = std::fopen(cache_path, "a");
        if (!f) return fail(GGDMC_ERR_ARG, std::string("cannot append to ") + cache_path);
        std::fprintf(f, "%s %d %d %d %d %.6f\n", key, t->spec_group, t->graph_iters, t->mig_round, t->lik_variant,
                     t->sweep_ms);
        std::fclose(f);
    }
    return GGDMC_OK;
}

ggdmc_status ggdmc_handle_set_tuning(ggdmc_handle *h, const ggdmc_tuning *t)
{
    if (!h) return fail(GGDMC_ERR_ARG, "handle is NULL");
    h->tuning = t ? *t : ggdmc_tuning{};
    return GGDMC_OK;
}

ggdmc_status ggdmc_autotune(ggdmc_handle *h, const ggdmc_de_config *cfg, const ggdmc_prior *p_prior,
                            const ggdmc_prior *h_prior, const ggdmc_chain_state *phi_state,
                            const ggdmc_chain_state *subj_state, int32_t n_probe, const char *cache_path,
                            ggdmc_tuning *out)
{
    if (!h || !cfg || !p_prior || !subj_state || n_probe < 1) return fail(GGDMC_ERR_ARG, "bad autotune arguments");
    if (h->S < 1) return fail(GGDMC_ERR_ARG, "handle has no subjects");
    ggdmc_status s;
    if ((s = check_cfg(cfg))) return s;
    // the key from the handle's own design and trial counts
    ggdmc_model m{};
    m.model_type = h->model_type;
    m.n_par = h->n_par;
    m.n_acc = h->n_acc;
    ggdmc_data d{};
    d.n_subject = h->S;
    d.offsets = h->h_offs.data();
    char key[512];
    if ((s = ggdmc_tune_key(&m, &d, cfg->nchain, phi_state != nullptr, key, sizeof key))) return s;
    ggdmc_tuning best{};
    if (!ggdmc_tune_lookup(key, cache_path, &best)) {
        h->tuning = best;
        if (out) *out = best;
        return GGDMC_OK;
    }
    g_err.clear();
    // probes: private copies of the start states, no samples kept
    const int S = h->S, C = cfg->nchain, P = h->n_par;
    std::vector<double> th((size_t)S * C * P), lp((size_t)S * C), ll((size_t)S * C);
    std::vector<double> pth(phi_state ? (size_t)C * 2 * P : 0), plp(phi_state ? C : 0), pll(phi_state ? C : 0);
    std::vector<ggdmc_chain_state> ss(S);
    ggdmc_chain_state ps{};
    ggdmc_de_config pc = *cfg;
    pc.nmc = n_probe + 1;
    pc.thin = 1;
    auto probe = [&](const ggdmc_tuning &t, double &ms) -> ggdmc_status {
        for (int l = 0; l < S; ++l) {
            std::memcpy(th.data() + (size_t)l * C * P, subj_state[l].theta, sizeof(double) * C * P);
            std::memcpy(lp.data() + (size_t)l * C, subj_state[l].lp, sizeof(double) * C);
            std::memcpy(ll.data() + (size_t)l * C, subj_state[l].ll, sizeof(double) * C);
            ss[l] = ggdmc_chain_state{th.data() + (size_t)l * C * P, lp.data() + (size_t)l * C, ll.data() + (size_t)l * C};
        }
        if (phi_state) {
            std::memcpy(pth.data(), phi_state->theta, sizeof(double) * pth.size());
            std::memcpy(plp.data(), phi_state->lp, sizeof(double) * C);
            std::memcpy(pll.data(), phi_state->ll, sizeof(double) * C);
            ps = ggdmc_chain_state{pth.data(), plp.data(), pll.data()};
        }
        h->tuning = t;
        ggdmc_run_stats st{};
        RunArgs a{phi_state ? RK_HIER : RK_SUBJECTS, &pc, p_prior, h_prior, phi_state ? &ps : nullptr, ss.data(),
                  nullptr, nullptr, nullptr, &st, nullptr, 0};
        ggdmc_status rs = run_impl(h, a);
        ms = st.sweep_ms / std::max<int64_t>(1, st.iterations);
        return rs;
    };
    // one setting at a time from the built-in choice; each probe runs twice
    // (the first warms the graph and caches) and the second time counts
    ggdmc_tuning cur{};
    double cur_ms = 0.0;
    auto measure = [&](const ggdmc_tuning &t, double &ms) -> ggdmc_status {
        double w = 0.0;
        ggdmc_status rs = probe(t, w);
        if (!rs) rs = probe(t, ms);
        return rs;
    };
    if ((s = measure(cur, cur_ms))) { h->tuning = ggdmc_tuning{}; return s; }
    auto consider = [&](ggdmc_tuning t) -> ggdmc_status {
        double ms = 0.0;
        ggdmc_status rs = measure(t, ms);
        if (rs) return rs;
        if (ms < cur_ms * 0.99) {
            cur = t;
            cur_ms = ms;
        }
        return GGDMC_OK;
    };
    auto tweak = [&](int32_t ggdmc_tuning::*f, int32_t v) -> ggdmc_status {
        ggdmc_tuning t = cur;
        t.*f = v;
        return consider(t);
    };
    if (h->model_type != GGDMC_MODEL_DDM && h->n_acc == 4) s = tweak(&ggdmc_tuning::lik_variant, 2);
    for (int g : {1, 2, 4}) if (!s) s = tweak(&ggdmc_tuning::spec_group, g);
    for (int mr : {3, 6, 8}) if (!s) s = tweak(&ggdmc_tuning::mig_round, mr);
    for (int gi : {4, 16}) if (!s) s = tweak(&ggdmc_tuning::graph_iters, gi);
    if (s) {
        h->tuning = ggdmc_tuning{};
        return s;
    }
    cur.sweep_ms = cur_ms;
    h->tuning = cur;
    if (out) *out = cur;
    return ggdmc_tune_store(key, cache_path, &cur);
}

}  // extern "C"
