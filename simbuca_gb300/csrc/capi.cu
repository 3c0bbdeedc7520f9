// capi.cu -- the extern "C" boundary of libsimgb (include/simgb.h): contexts, device
// state of resident clouds, work planning, CUDA-graph replay of the Dormand-Prince
// attempt, stand-alone force calls and the CUNBODY-compatible slot.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "sg_internal.cuh"
#include "sg_mt19937.h"

namespace {

// ---------------------------------------------------------------------------
// Device state of a set of clouds (a batch; a stand-alone call uses a batch of one).
// ---------------------------------------------------------------------------
struct Problem {
    int n_clouds = 0, n = 0, npad = 0, precision = 0, n_rows = 0, n_items = 0, max_slots = 0;
    int variant = 0;  // FP32c launch shape the items were planned for
    int method = 5;   // 5 Dormand-Prince, 4 Cash-Karp (every cloud of a batch)
    bool any_coulomb = false;
    bool uploaded = false;
    std::vector<SgCloud> hc;
    std::vector<SgCtrl> hctrl0;
    std::vector<SgRowBlock> hrows;
    std::vector<SgWorkItem> hitems;
    std::vector<int> counts;
    SgCloud* dc = nullptr;
    SgCtrl* dctrl = nullptr;
    SgRowBlock* drows = nullptr;
    SgWorkItem* ditems = nullptr;
    double *y = nullptr, *ys = nullptr, *k = nullptr, *part = nullptr, *coul1 = nullptr,
           *coul7 = nullptr, *coulS = nullptr, *kq = nullptr, *qm = nullptr, *qd = nullptr, *mass = nullptr,
           *c64 = nullptr, *err_part = nullptr, *mom = nullptr, *stage = nullptr;
    float* c32 = nullptr;
    int* flags = nullptr;  // [0] error word, [1] hold-on-accept, [2] FP32c fix-up count
    SgCtrl* hctrl = nullptr;  // pinned mirror of dctrl
    double interactions = 0.0;  // per Coulomb evaluation, all clouds
    std::vector<double> cloud_inter;
    // ion order: device arrays hold ions in k-d tree order when `sorted`; perm maps a
    // device position to the caller's ion index
    bool sorted = false;
    std::vector<int> perm;
    int* dperm = nullptr;
    float* bbox = nullptr;        // [ntiles][8]
    int ntiles = 0;
    double *kq0 = nullptr, *qm0 = nullptr, *qd0 = nullptr, *mass0 = nullptr;  // caller order
    // learned step-size proposer and step-history log
    SgProposerState* pst = nullptr;
    void* wbf = nullptr;           // BF16 MLP weights
    float* log_feat = nullptr;     // [clouds][log_cap][16]
    double* log_num = nullptr;     // [clouds][log_cap][4]: h_prev, h, err, t
    int log_cap = 0;
    int use_mlp = 0;
    double safety = 0.9;
    // recorder (device-side observables): rings of records per cloud, drained into
    // host memory whenever the host synchronises
    double* ring = nullptr;
    int* spec0 = nullptr;  // species per ion, caller order
    int* spec = nullptr;   // species per ion, device order
    int n_species = 1, rec_stride = 1, rec_cap = 0;
    double print_interval = 0.0;
    std::vector<std::vector<double>> rec_host;
    std::vector<int> hspec0;
    std::vector<double> hmass0;
    double *pmass = nullptr, *pmass0 = nullptr;  // print masses (dissociation), both orders
    int* fix_list = nullptr;   // FP32c fix-up work lists: counts, then (ion, cloud) pairs
    double* fix_part = nullptr;  // fix-up work units' corrections [listed][units][3]
    int* fix_done = nullptr;     // finished units per listed ion (zero between calls)
    // operation sequence
    std::vector<sg_field_params> fp0;  // field parameters as created / set by the caller
    std::vector<SgOp> hops;
    SgOp* dops = nullptr;
    int* dis_spec = nullptr;     // [dissociations][N] caller order
    double* dis_mass = nullptr;
    int n_dis = 0;
    // in-run force check of the FP32c sums (check.cu): every check_every attempts
    float* risk = nullptr;   // [2][N] far and near ratios of the last in-attempt sum
    int* ran = nullptr;      // [clouds] an in-attempt sum ran since the last check
    SgCheck* dchk = nullptr; // [clouds] check records and measured thresholds
    int check_every = 16;
    long long attempt_count = 0;
    double kfar_prior = 0.0;  // > 0: the far fix-up threshold's prior of every cloud
    // fused small-cloud attempts (fused.cu)
    double* errp = nullptr;   // [clouds][SG_FUSED_MAX_CTAS]
    int fused_cluster = -1;   // cluster size for this batch (0: not launchable), -1 unknown
    int max_npad = 0;         // largest padded cloud
};

struct TimedLaunch {
    cudaEvent_t a, b;
    double inter;
    int fused;  // a fused-attempts launch (else a Coulomb pair kernel)
};

}  // namespace

// O(N) kernels of one attempt timed by the kernel-timing graph (at most)
constexpr int kStageMarks = 12;

// Launches may use programmatic dependent launch (sg_launch): set while the untimed
// attempt graph is captured when SIMGB_PDL=1 is in the environment.  Off by default: on
// GB300 it gave +2.8 % on a 1,000-ion FP32c cloud but halved the plain FP64 form's rate
// on 4,096 ions (its Coulomb kernel unchanged; the cause is not known).
int g_sg_pdl = 0;

struct sg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    int last_err = 0;
    int n_sm = 148;
    int c32_variant = -1;  // -1: chosen per batch from the cloud sizes
    Problem batch;
    Problem solo;
    bool timing = false;
    std::vector<TimedLaunch> pending;
    std::vector<cudaEvent_t> free_ev;
    double coul_ms = 0.0, coul_inter = 0.0;
    long long coul_launches = 0;
    double fused_ms = 0.0;
    long long fused_launches = 0;
    int use_fused = 1;  // 0 off, 1 clouds up to SG_FUSED_AUTO_IONS, 2 up to SG_FUSED_MAX_IONS
    bool use_graph = true;
    cudaGraphExec_t graph = nullptr;
    // timed graph: the same attempt with an event pair around each Coulomb launch
    cudaGraphExec_t graph_timed = nullptr;
    cudaEvent_t gev[16] = {nullptr};
    int capture_events = -1;  // next event pair while capturing the timed graph, else -1
    // the same for the O(N) kernels of an attempt (stages, control, commit)
    cudaEvent_t sev[2 * kStageMarks] = {nullptr};
    int capture_stage = -1;
    int stage_pairs = 0;  // pairs recorded by the timed graph
    double stage_ms = 0.0;
    long long stage_launches = 0;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    int* herr = nullptr;  // pinned host word for the device error word
    float* probe_sink = nullptr;
    // MLP training buffers
    float *mlp_wm = nullptr, *mlp_m1 = nullptr, *mlp_m2 = nullptr, *mlp_grad = nullptr,
          *mlp_gpart = nullptr, *mlp_lpart = nullptr, *mlp_loss = nullptr, *mlp_X = nullptr,
          *mlp_Y = nullptr, *mlp_out = nullptr;
    int* mlp_idx = nullptr;
    void* mlp_wbf = nullptr;
    int mlp_cap = 0;
    // CUNBODY slot buffers
    double *cb_xj = nullptr, *cb_mj = nullptr, *cb_xi = nullptr, *cb_ai = nullptr;
    double* cb_host = nullptr;
    int cb_ni = 0, cb_nj = 0;
};

namespace {

#define CK(call)                                   \
    do {                                           \
        cudaError_t e_ = (call);                   \
        if (e_ != cudaSuccess) {                   \
            ctx->last_err = (int)e_;               \
            return SG_CUDA_ERR;                    \
        }                                          \
    } while (0)

template <typename T>
cudaError_t dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void**)p, count * sizeof(T));
}

void free_problem(Problem& P) {
    cudaFree(P.dc);
    cudaFree(P.dctrl);
    cudaFree(P.drows);
    cudaFree(P.ditems);
    double* ds[] = {P.y, P.ys, P.k, P.part, P.coul1, P.coul7, P.coulS, P.kq, P.qm,
                    P.qd, P.mass, P.c64, P.err_part, P.mom, P.stage};
    for (double* d : ds) cudaFree(d);
    cudaFree(P.c32);
    cudaFree(P.flags);
    cudaFree(P.pst);
    cudaFree(P.wbf);
    cudaFree(P.dperm);
    cudaFree(P.ring);
    cudaFree(P.spec0);
    cudaFree(P.spec);
    cudaFree(P.pmass);
    cudaFree(P.pmass0);
    cudaFree(P.fix_list);
    cudaFree(P.fix_part);
    cudaFree(P.fix_done);
    cudaFree(P.dops);
    cudaFree(P.dis_spec);
    cudaFree(P.dis_mass);
    cudaFree(P.bbox);
    cudaFree(P.kq0);
    cudaFree(P.qm0);
    cudaFree(P.qd0);
    cudaFree(P.mass0);
    cudaFree(P.log_feat);
    cudaFree(P.log_num);
    cudaFree(P.risk);
    cudaFree(P.ran);
    cudaFree(P.dchk);
    cudaFree(P.errp);
    if (P.hctrl) cudaFreeHost(P.hctrl);
    P = Problem();
}

inline int round_up(int a, int b) { return (a + b - 1) / b * b; }

// Thresholds from the launch-shape tuner (simbuca_gb300/tune.py) on GB300: one cloud of
// up to ~6k ions is latency-bound and runs best as one-warp blocks of 32 ions (11);
// 64 x 2 blocks (5) to ~24k; the k-d ordered shapes beyond (9; 14 from ~48k).  A batch
// whose pair work fills the GPU on its own (the 512-cloud scan: 3.5e9 pairs per call)
// takes the k-d ordered leaf shape whatever its largest cloud.
int auto_variant(const std::vector<int>& counts, int requested) {
    if (requested >= 0) return requested;
    int big = 0;
    double pairs = 0.0;
    for (int n : counts) {
        big = std::max(big, n);
        pairs += (double)n * (double)n;
    }
    if (big >= 48000) return 14;
    if (pairs >= 2e9) return 9;
    if (big <= 6000) return 11;
    return big < 24000 ? 5 : 9;
}

// Partition clouds into row blocks and Coulomb work items.  Items are sized so that
// (a) there are several waves of blocks on the device and (b) no single item is a
// large share of the total work; they are issued largest first.
void plan(Problem& P, int n_sm) {
    const int C = P.n_clouds;
    std::vector<sg_field_params> fps(C);
    for (int c = 0; c < C; c++) fps[c] = P.hc[c].fp;  // callers set the field terms first
    P.hc.assign(C, SgCloud());
    P.hrows.clear();
    P.hitems.clear();
    P.cloud_inter.assign(C, 0.0);
    int off = 0, poff = 0, tiles = 0;
    P.any_coulomb = false;
    P.sorted = P.precision == SG_PREC_FP32C && sg_variant_sorted(P.variant);
    // Row blocks of SG_ROWS ions, or fewer for small batches: the stage, control and
    // reduction kernels are FP64 work, which GB300 runs at a small fraction of its FP32
    // rate per SM, so a 1,000-ion cloud is spread over 32 SMs rather than 4.  The k-d
    // ordered shapes keep full blocks (each covers two 128-ion tiles for the tile bounds).
    long long total_ions = 0;
    for (int c = 0; c < C; c++) total_ions += P.counts[c];
    int rows = SG_ROWS;
    if (!P.sorted)
        while (rows > 32 && total_ions / rows < 2LL * n_sm) rows /= 2;
    for (int c = 0; c < C; c++) {
        SgCloud& cl = P.hc[c];
        memset(&cl, 0, sizeof cl);
        cl.qscale = 1.0;
        cl.fp = fps[c];
        cl.off = off;
        cl.n = P.counts[c];
        cl.poff = poff;
        cl.npad = round_up(cl.n, SG_PAD);
        cl.tile0 = tiles;
        tiles += (cl.npad + 127) / 128;
        cl.rb0 = (int)P.hrows.size();
        for (int i = 0; i < cl.n; i += rows) {
            SgRowBlock rb;
            rb.cloud = c;
            rb.i0 = off + i;
            rb.n = std::min(rows, cl.n - i);
            rb.pad = 0;
            P.hrows.push_back(rb);
        }
        cl.nrb = (int)P.hrows.size() - cl.rb0;
        off += cl.n;
        poff += cl.npad;
    }
    P.n = off;
    P.npad = poff;
    P.ntiles = tiles;
    P.n_rows = (int)P.hrows.size();

    const bool f32 = P.precision == SG_PREC_FP32C;
    const int ib = f32 ? sg_coulomb_fp32c_ib(P.variant) : SG_C64_IB;
    const int per_sm = f32 ? std::max(1, 2048 / ib) : 4;
    const double conc = (double)n_sm * per_sm;
    double total = 0.0;
    for (int c = 0; c < C; c++)
        if (P.hc[c].fp.flags & SG_F_COULOMB) total += (double)P.hc[c].n * P.hc[c].npad;
    std::vector<int> S(C, 0);
    long long items = 0;
    const double cap = std::max(total / (conc * 2.0), 512.0 * 512.0);
    for (int c = 0; c < C; c++) {
        const SgCloud& cl = P.hc[c];
        if (!(cl.fp.flags & SG_F_COULOMB) || cl.n == 0) continue;
        const double jmax = std::max(128.0, std::floor(cap / std::min(ib, cl.n) / 128.0) * 128.0);
        S[c] = std::max(1, (int)std::ceil(cl.npad / jmax));
        items += (long long)((cl.n + ib - 1) / ib) * S[c];
    }
    // j-chunks are whole 128-ion tiles, or smaller ones (plain shapes only: the k-d
    // ordered kernels test whole tiles) when 128-ion chunks would leave fewer than two
    // blocks per SM.  FP32c: 64-ion chunks -- a 1,000-ion cloud runs 512 one-warp blocks
    // instead of 256 (7 % faster per step than 32-ion chunks, whose 32 partial-sum slots
    // made the reduction dearer than the extra parallelism paid).  FP64: 32-ion chunks,
    // its pair kernel being bound by the FP64 pipe of every SM it can reach (1,000 ions:
    // 23 sim-us/s with 32-ion chunks, 14.5 with 64).
    long long full_split = 0;
    for (int c = 0; c < C; c++)
        if (S[c] > 0)
            full_split += (long long)((P.hc[c].n + ib - 1) / ib) * std::max(1, P.hc[c].npad / 128);
    const int jgran = (!P.sorted && full_split < 2LL * n_sm) ? (f32 ? 64 : 32) : 128;
    const double target = conc * 4.0;
    if (items > 0 && items < target) {
        const int f = (int)std::ceil(target / (double)items);
        for (int c = 0; c < C; c++)
            if (S[c] > 0) S[c] = std::min(S[c] * f, std::max(1, P.hc[c].npad / jgran));
    }
    P.max_slots = 0;
    for (int c = 0; c < C; c++) {
        SgCloud& cl = P.hc[c];
        if (S[c] == 0) {
            cl.nslots = 0;
            continue;
        }
        P.any_coulomb = true;
        const int jc = round_up((cl.npad + S[c] - 1) / S[c], jgran);
        int slot = 0;
        for (int j0 = 0; j0 < cl.npad; j0 += jc, slot++) {
            const int nj = std::min(jc, cl.npad - j0);
            for (int i = 0; i < cl.n; i += ib) {
                SgWorkItem it;
                memset(&it, 0, sizeof it);
                it.cloud = c;
                it.i0 = cl.poff + i;
                it.ni = std::min(ib, cl.n - i);
                it.j0 = cl.poff + j0;
                it.nj = nj;
                it.slot = slot;
                P.hitems.push_back(it);
            }
        }
        cl.nslots = slot;
        P.max_slots = std::max(P.max_slots, slot);
        P.cloud_inter[c] = (double)cl.n * (cl.n - 1);
    }
    std::stable_sort(P.hitems.begin(), P.hitems.end(), [](const SgWorkItem& a, const SgWorkItem& b) {
        return (long long)a.ni * a.nj > (long long)b.ni * b.nj;
    });
    P.n_items = (int)P.hitems.size();
}

// FP32 frame of a cloud: centre = centroid, L = largest per-axis RMS spread; the
// close-pair threshold wc = 1/rc^3 with rc = 0.6 x the mean ion spacing of a Gaussian
// cloud of the same spreads, in frame units.
void set_frame(SgCloud& cl, const double* pos_aos, int off) {
    const int n = cl.n;
    double m[3] = {0, 0, 0}, v[3] = {0, 0, 0};
    for (int i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) m[c] += pos_aos[3 * (size_t)(off + i) + c];
    for (int c = 0; c < 3; c++) m[c] = n ? m[c] / n : 0.0;
    for (int i = 0; i < n; i++)
        for (int c = 0; c < 3; c++) {
            const double d = pos_aos[3 * (size_t)(off + i) + c] - m[c];
            v[c] += d * d;
        }
    double s[3], L = 0.0;
    for (int c = 0; c < 3; c++) {
        s[c] = n ? std::sqrt(v[c] / n) : 0.0;
        L = std::max(L, s[c]);
    }
    if (!(L > 0.0) || !std::isfinite(L)) L = 1e-3;
    cl.cx = m[0];
    cl.cy = m[1];
    cl.cz = m[2];
    cl.L = L;
    cl.invL = 1.0 / L;
    double vol = std::pow(2.0 * SG_PI, 1.5);
    for (int c = 0; c < 3; c++) vol *= std::max(s[c] / L, 1e-3);
    const double spacing = std::cbrt(vol / std::max(n, 1));
    const double rc = 0.6 * spacing;
    cl.wc = (float)(1.0 / (rc * rc * rc));
    // far tiles (sorted kernel): beyond every capped pair, and far enough that the
    // high parts alone give the pair distance to ~1e-6
    cl.dfar = (float)std::max(0.25, 1.01 * rc);
    // Prior of the far fix-up threshold.  The error of the hi-only far terms is
    // ~c sqrt(s2f)/|P| with c growing with the ion density in frame units, n / vol.
    // Measured (numpy model of the kernel's arithmetic, and the GPU): c = 2.5e-7 for the
    // 65,536-ion Gaussian cloud (density 4.2e3), 1.2e-6 for the 1M-ion uniform spheroid
    // (density 2.7e5): c = 1.08e-8 density^0.377 through both.  Ions with
    // c sqrt(s2f) > 5e-7 |P| are fixed up, which keeps the others at half the 1e-6 bound.
    // The in-run check (check.cu) measures c on the cloud itself and lowers the
    // threshold when it finds a larger c.
    const double density = std::max(n, 1) / vol;
    const double c_far = 1.08e-8 * std::pow(density, 0.377);
    const double kfar = 5e-7 / c_far;
    cl.kfar2 = (float)(kfar * kfar);
}

// k-d tree order of one cloud: recursive median splits along the widest axis, the
// lower part always a multiple of 128 ions, so that every 128-ion tile is a leaf.
void kd_order(const double* pos, int off, int n, int* out) {
    std::vector<int> idx(n);
    for (int i = 0; i < n; i++) idx[i] = off + i;
    std::vector<std::pair<int, int>> stack;
    stack.push_back(std::make_pair(0, n));
    while (!stack.empty()) {
        const int b = stack.back().first, e = stack.back().second;
        stack.pop_back();
        const int len = e - b;
        if (len <= 128) continue;
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int i = b; i < e; i++)
            for (int c = 0; c < 3; c++) {
                const double v = pos[3 * (size_t)idx[i] + c];
                lo[c] = std::min(lo[c], v);
                hi[c] = std::max(hi[c], v);
            }
        int ax = 0;
        for (int c = 1; c < 3; c++)
            if (hi[c] - lo[c] > hi[ax] - lo[ax]) ax = c;
        const int m = std::min(len - 1, (len / 2 + 127) / 128 * 128);
        std::nth_element(idx.begin() + b, idx.begin() + b + m, idx.begin() + e,
                         [pos, ax](int p, int q) { return pos[3 * (size_t)p + ax] < pos[3 * (size_t)q + ax]; });
        stack.push_back(std::make_pair(b + m, e));
        stack.push_back(std::make_pair(b, b + m));
    }
    for (int i = 0; i < n; i++) out[i] = idx[i];
}

int alloc_problem(sg_ctx* ctx, Problem& P) {
    const size_t N = (size_t)std::max(P.n, 1), NP = (size_t)std::max(P.npad, 1);
    CK(dalloc(&P.dc, (size_t)std::max(P.n_clouds, 1)));
    CK(dalloc(&P.dctrl, (size_t)std::max(P.n_clouds, 1)));
    CK(dalloc(&P.drows, (size_t)std::max(P.n_rows, 1)));
    CK(dalloc(&P.ditems, (size_t)std::max(P.n_items, 1)));
    CK(dalloc(&P.y, 6 * N));
    CK(dalloc(&P.ys, 6 * N));
    CK(dalloc(&P.k, 42 * N));
    CK(dalloc(&P.part, (size_t)std::max(P.max_slots, 1) * SG_PART_ARRAYS * NP));
    CK(dalloc(&P.coulS, 3 * N));
    CK(dalloc(&P.coul1, 3 * N));
    CK(dalloc(&P.coul7, 3 * N));
    CK(dalloc(&P.kq, N));
    CK(dalloc(&P.qm, N));
    CK(dalloc(&P.qd, N));
    CK(dalloc(&P.mass, N));
    CK(dalloc(&P.c64, 4 * NP));
    CK(dalloc(&P.c32, 7 * NP));
    CK(dalloc(&P.err_part, (size_t)std::max(P.n_rows, 1)));
    CK(dalloc(&P.mom, (size_t)std::max(P.n_rows, 1) * 11));
    CK(dalloc(&P.stage, 6 * N));
    CK(dalloc(&P.flags, SG_NFLAGS));
    CK(cudaMemset(P.flags, 0, SG_NFLAGS * sizeof(int)));
    CK(dalloc(&P.errp, (size_t)std::max(P.n_clouds, 1) * SG_FUSED_MAX_CTAS));
    P.max_npad = 0;
    for (int c = 0; c < P.n_clouds; c++) P.max_npad = std::max(P.max_npad, P.hc[c].npad);
    if (P.precision == SG_PREC_FP32C) {
        CK(dalloc(&P.risk, 2 * N));
        CK(dalloc(&P.ran, (size_t)std::max(P.n_clouds, 1)));
        CK(cudaMemset(P.ran, 0, sizeof(int) * (size_t)std::max(P.n_clouds, 1)));
        std::vector<SgCheck> h0((size_t)std::max(P.n_clouds, 1));
        for (SgCheck& h : h0) {
            memset(&h, 0, sizeof h);
            h.kfar2 = INFINITY;
        }
        CK(dalloc(&P.dchk, h0.size()));
        CK(cudaMemcpy(P.dchk, h0.data(), sizeof(SgCheck) * h0.size(), cudaMemcpyHostToDevice));
    }
    CK(dalloc(&P.pst, (size_t)std::max(P.n_clouds, 1)));
    CK(cudaMemset(P.pst, 0, sizeof(SgProposerState) * (size_t)std::max(P.n_clouds, 1)));
    CK(cudaMalloc(&P.wbf, SG_MLP_NP * 2));
    CK(cudaMemset(P.wbf, 0, SG_MLP_NP * 2));
    CK(dalloc(&P.dperm, N));
    CK(dalloc(&P.spec0, N));
    CK(dalloc(&P.spec, N));
    CK(cudaMemset(P.spec0, 0, N * sizeof(int)));
    CK(cudaMemset(P.spec, 0, N * sizeof(int)));
    CK(dalloc(&P.pmass, N));
    CK(dalloc(&P.pmass0, N));
    // two lists (near-only ions; ions with a far fix-up): counts, then N pairs each
    CK(dalloc(&P.fix_list, 2 + 4 * N));
    CK(cudaMemset(P.fix_list, 0, 2 * sizeof(int)));
    // two lists (row re-evaluations, far corrections) of up to SG_FIX_CHUNKED_CAP ions
    CK(dalloc(&P.fix_part, (size_t)2 * SG_FIX_CHUNKED_CAP * SG_FIX_UNITS * 3));
    CK(dalloc(&P.fix_done, 2 * SG_FIX_CHUNKED_CAP));
    CK(cudaMemset(P.fix_done, 0, sizeof(int) * 2 * SG_FIX_CHUNKED_CAP));
    CK(cudaMemset(P.pmass, 0, N * sizeof(double)));
    CK(cudaMemset(P.pmass0, 0, N * sizeof(double)));
    CK(dalloc(&P.bbox, (size_t)std::max(P.ntiles, 1) * 8));
    CK(dalloc(&P.kq0, N));
    CK(dalloc(&P.qm0, N));
    CK(dalloc(&P.qd0, N));
    CK(dalloc(&P.mass0, N));
    CK(cudaMemset(P.mass0, 0, N * sizeof(double)));
    CK(cudaMemset(P.qm0, 0, N * sizeof(double)));
    P.perm.resize(P.n);
    for (int i = 0; i < P.n; i++) P.perm[i] = i;
    CK(cudaMemcpy(P.dperm, P.perm.data(), sizeof(int) * P.n, cudaMemcpyHostToDevice));
    CK(cudaMemset(P.coul1, 0, 3 * N * sizeof(double)));
    CK(cudaMemset(P.part, 0, (size_t)std::max(P.max_slots, 1) * SG_PART_ARRAYS * NP * sizeof(double)));
    CK(cudaMemset(P.coulS, 0, 3 * N * sizeof(double)));
    CK(cudaMallocHost((void**)&P.hctrl, sizeof(SgCtrl) * (size_t)std::max(P.n_clouds, 1)));
    CK(cudaMemcpy(P.drows, P.hrows.data(), sizeof(SgRowBlock) * P.hrows.size(),
                  cudaMemcpyHostToDevice));
    if (P.n_items)
        CK(cudaMemcpy(P.ditems, P.hitems.data(), sizeof(SgWorkItem) * P.hitems.size(),
                      cudaMemcpyHostToDevice));
    return SG_OK;
}

SgDpArgs dp_args(Problem& P) {
    SgDpArgs a;
    a.rows = P.drows;
    a.clouds = P.dc;
    a.ctrl = P.dctrl;
    a.y = P.y;
    a.ys = P.ys;
    a.k = P.k;
    a.coulS = P.coulS;
    a.coul1 = P.coul1;
    a.coul7 = P.coul7;
    a.kq = P.kq;
    a.qm = P.qm;
    a.c64 = P.c64;
    a.c32 = P.c32;
    a.err_part = P.err_part;
    a.bbox = P.sorted ? P.bbox : nullptr;
    a.n = P.n;
    a.npad = P.npad;
    a.fp32c = P.precision == SG_PREC_FP32C ? 1 : 0;
    return a;
}

// Host copy of the per-cloud records, field parameters included, from the device.
cudaError_t pull_clouds(sg_ctx* ctx, Problem& P) {
    cudaError_t e = cudaMemcpyAsync(P.hc.data(), P.dc, sizeof(SgCloud) * P.n_clouds,
                                    cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(ctx->stream);
}

// Species and print masses after each dissociation of the sequence, caller order: per
// cloud the reference's loop over its ions (bin/operation.cpp:59-70) with MTRand seeded
// 0 at each dissociation, one draw per ion of the reactant species.
int dissociation_tables(sg_ctx* ctx, Problem& P) {
    int n_dis = 0;
    for (const SgOp& op : P.hops)
        if (op.kind == SG_OP_DISSOCIATION) n_dis++;
    cudaFree(P.dis_spec);
    cudaFree(P.dis_mass);
    P.dis_spec = nullptr;
    P.dis_mass = nullptr;
    P.n_dis = n_dis;
    if (n_dis == 0) return SG_OK;
    const size_t N = (size_t)P.n;
    std::vector<int> spec(P.hspec0);
    std::vector<double> mass(P.hmass0);
    std::vector<int> ts(N * n_dis);
    std::vector<double> tm(N * n_dis);
    int d = 0;
    for (const SgOp& op : P.hops) {
        if (op.kind != SG_OP_DISSOCIATION) continue;
        for (int c = 0; c < P.n_clouds; c++) {
            SgMt19937 rng(0u);
            for (int i = P.hc[c].off; i < P.hc[c].off + P.hc[c].n; i++)
                if (spec[i] == op.reactant && rng.uniform() < op.fraction) {
                    spec[i] = op.product;
                    mass[i] = op.product_mass;
                }
        }
        std::copy(spec.begin(), spec.end(), ts.begin() + d * N);
        std::copy(mass.begin(), mass.end(), tm.begin() + d * N);
        d++;
    }
    CK(dalloc(&P.dis_spec, N * n_dis));
    CK(dalloc(&P.dis_mass, N * n_dis));
    CK(cudaMemcpyAsync(P.dis_spec, ts.data(), sizeof(int) * ts.size(), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemcpyAsync(P.dis_mass, tm.data(), sizeof(double) * tm.size(), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

SgRecArgs rec_args(Problem& P) {
    SgRecArgs r;
    r.rows = P.drows;
    r.clouds = P.dc;
    r.ctrl = P.dctrl;
    r.y = P.y;
    r.mass = P.pmass;
    r.spec = P.spec;
    r.dis_spec = P.dis_spec;
    r.dis_mass = P.dis_mass;
    r.perm = P.dperm;
    r.ring = P.ring;
    r.n = P.n;
    r.n_species = P.n_species;
    r.stride = P.rec_stride;
    return r;
}

// Moves the records written since the last drain into host memory and lets clouds held
// by a full ring go on.  The stream must be idle and hctrl current (after sync_ctrl).
int drain_records(sg_ctx* ctx, Problem& P) {
    if (P.rec_cap <= 0) return SG_OK;
    bool changed = false;
    for (int c = 0; c < P.n_clouds; c++) {
        SgCtrl& s = P.hctrl[c];
        const SgCloud& cl = P.hc[c];
        const long long k = s.rec_count - s.rec_drained;
        if (k <= 0 && !(s.hold & 2)) continue;
        std::vector<double>& dst = P.rec_host[c];
        for (long long r = s.rec_drained; r < s.rec_count; r++) {
            const size_t at = dst.size();
            dst.resize(at + cl.rec_len);
            const double* src = P.ring + cl.rec_off + (r % P.rec_cap) * (long long)cl.rec_len;
            CK(cudaMemcpyAsync(dst.data() + at, src, sizeof(double) * cl.rec_len,
                               cudaMemcpyDeviceToHost, ctx->stream));
        }
        s.rec_drained = s.rec_count;
        s.hold &= ~2;
        changed = true;
    }
    if (changed) {
        CK(cudaMemcpyAsync(P.dctrl, P.hctrl, sizeof(SgCtrl) * P.n_clouds, cudaMemcpyHostToDevice,
                           ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return SG_OK;
}

cudaEvent_t take_event(sg_ctx* ctx) {
    if (!ctx->free_ev.empty()) {
        cudaEvent_t e = ctx->free_ev.back();
        ctx->free_ev.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// Accumulate the finished timed launches (call after the stream is synchronised).
void flush_timing(sg_ctx* ctx) {
    for (auto& tl : ctx->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, tl.a, tl.b) == cudaSuccess) {
            if (tl.fused) {
                ctx->fused_ms += ms;
                ctx->fused_launches += 1;
            } else {
                ctx->coul_ms += ms;
                ctx->coul_launches += 1;
                ctx->coul_inter += tl.inter;
            }
        }
        ctx->free_ev.push_back(tl.a);
        ctx->free_ev.push_back(tl.b);
    }
    ctx->pending.clear();
}

// Coulomb sums of the current Coulomb inputs into out[3][N]: the pair kernel over the
// work items, then the per-ion reduction of the partial-sum slots (with the FP32c
// conditioning fix-up).
// far_estimate: recompute the far tiles' conditioning estimate in this call (the first
// Coulomb sum of an attempt and every stand-alone one); later stages of the attempt
// reuse it -- the ions barely move within a step, and only the choice of which ions to
// fix up depends on it.
int launch_coulomb(sg_ctx* ctx, Problem& P, bool with_ctrl, double inter, double* out,
                   bool far_estimate = true) {
    if (!P.any_coulomb || P.n_items == 0) return SG_OK;
    SgCoulombArgs ca;
    ca.c32 = P.c32;
    ca.c64 = P.c64;
    ca.items = P.ditems;
    ca.n_items = P.n_items;
    ca.clouds = P.dc;
    ca.ctrl = with_ctrl ? P.dctrl : nullptr;
    ca.part = P.part;
    ca.npad_total = P.npad;
    ca.errword = P.flags;
    ca.variant = P.variant;
    ca.bbox = P.bbox;
    ca.fix_list = P.fix_list;
    ca.fix_part = P.fix_part;
    ca.fix_done = P.fix_done;
    ca.far_estimate = far_estimate ? 1 : 0;
    if (P.precision == SG_PREC_FP32C) {
        ca.chk = P.dchk;
        if (out == P.coulS) {
            ca.risk = P.risk;
            ca.ran = P.ran;
        }
    }
    TimedLaunch tl{nullptr, nullptr, inter, 0};
    const int cap = ctx->capture_events;
    if (cap >= 0) {
        // external event nodes: recorded by each replay and readable from the host
        CK(cudaEventRecordWithFlags(ctx->gev[2 * cap], ctx->stream, cudaEventRecordExternal));
    } else if (ctx->timing) {
        tl.a = take_event(ctx);
        tl.b = take_event(ctx);
        CK(cudaEventRecord(tl.a, ctx->stream));
    }
    const bool f32 = P.precision == SG_PREC_FP32C;
    if (f32)
        CK(sg_launch_coulomb_fp32c(ca, ctx->stream));
    else
        CK(sg_launch_coulomb_fp64(ca, ctx->stream));
    if (cap >= 0) {
        CK(cudaEventRecordWithFlags(ctx->gev[2 * cap + 1], ctx->stream, cudaEventRecordExternal));
        ctx->capture_events = cap + 1;
    } else if (ctx->timing) {
        CK(cudaEventRecord(tl.b, ctx->stream));
        ctx->pending.push_back(tl);
    }
    CK(sg_launch_coulomb_reduce(ca, P.drows, P.n_rows, f32 ? 1 : 0, out, P.n, P.flags + 2,
                                ctx->stream));
    return SG_OK;
}

// Interactions of the clouds that are still active (host view of the last sync).
double active_interactions(Problem& P) {
    double s = 0.0;
    for (int c = 0; c < P.n_clouds; c++)
        if (!P.hctrl[c].done && P.hctrl[c].status == SG_OK) s += P.cloud_inter[c];
    return s;
}

// External event pair around an O(N) kernel while the timed graph is being captured.
int stage_mark(sg_ctx* ctx, bool end) {
    const int k = ctx->capture_stage;
    if (k < 0 || k >= kStageMarks) return SG_OK;
    CK(cudaEventRecordWithFlags(ctx->sev[2 * k + (end ? 1 : 0)], ctx->stream,
                                cudaEventRecordExternal));
    if (end) ctx->capture_stage = k + 1;
    return SG_OK;
}

#define STAGE_TIMED(call)                          \
    do {                                           \
        int s_ = stage_mark(ctx, false);           \
        if (s_ != SG_OK) return s_;                \
        CK(call);                                  \
        s_ = stage_mark(ctx, true);                \
        if (s_ != SG_OK) return s_;                \
    } while (0)

// One Dormand-Prince attempt of every active cloud (bin/ode.cpp:61-218, 426-494).
int enqueue_attempt(sg_ctx* ctx, Problem& P) {
    SgDpArgs a = dp_args(P);
    const double inter = ctx->timing ? active_interactions(P) : 0.0;
    if (P.method == 1) {
        // Gear: predict, one force evaluation at the predicted state, correct
        STAGE_TIMED(sg_gear_stage(a, 0, P.n_rows, ctx->stream));
        int st = launch_coulomb(ctx, P, true, inter, P.coulS);
        if (st != SG_OK) return st;
        STAGE_TIMED(sg_gear_stage(a, 1, P.n_rows, ctx->stream));
    } else if (P.method == 4) {
        // Cash-Karp: the step start is no stage of the previous step, so its Coulomb
        // inputs are rebuilt and all six stages take a Coulomb sum
        STAGE_TIMED(sg_coords_from_state(a, P.qd, P.n_rows, ctx->stream));
        for (int s = 1; s <= 6; s++) {
            int st = launch_coulomb(ctx, P, true, inter, P.coulS, s == 1);
            if (st != SG_OK) return st;
            STAGE_TIMED(sg_ck_stage(a, s, P.n_rows, ctx->stream));
        }
    } else {
        STAGE_TIMED(sg_dp_stage(a, 1, P.n_rows, ctx->stream));
        for (int s = 2; s <= 7; s++) {
            int st = launch_coulomb(ctx, P, true, inter, P.coulS, s == 2);
            if (st != SG_OK) return st;
            STAGE_TIMED(sg_dp_stage(a, s, P.n_rows, ctx->stream));
        }
    }
    STAGE_TIMED(sg_dp_control(P.dc, P.dctrl, P.err_part, P.y, P.n_clouds, P.flags, P.dops,
                              ctx->stream));
    STAGE_TIMED(sg_dp_commit(a, P.n_rows, ctx->stream));
    if (P.rec_cap > 0) CK(sg_record(rec_args(P), P.n_rows, P.n_clouds, ctx->stream));
    if (P.n_dis > 0)
        CK(sg_dissociate(rec_args(P), P.pmass, P.spec0, P.pmass0, P.n_rows, ctx->stream));
    if (P.log_cap > 0 || P.use_mlp) {
        CK(sg_moments(a, P.mass, P.mom, P.n_rows, ctx->stream));
        CK(sg_proposer_launch(P.dc, P.dctrl, P.mom, P.pst, P.wbf, P.log_feat, P.log_num,
                              P.log_cap, P.use_mlp, P.safety, P.n_clouds, ctx->stream));
    }
    return SG_OK;
}

// Proposer state of a freshly uploaded state: features of the first step.
int proposer_reset(sg_ctx* ctx, Problem& P) {
    CK(cudaMemsetAsync(P.pst, 0, sizeof(SgProposerState) * P.n_clouds, ctx->stream));
    if (P.log_cap > 0 || P.use_mlp) {
        SgDpArgs a = dp_args(P);
        CK(sg_moments(a, P.mass, P.mom, P.n_rows, ctx->stream));
        CK(sg_proposer_launch(P.dc, P.dctrl, P.mom, P.pst, P.wbf, P.log_feat, P.log_num,
                              P.log_cap, P.use_mlp, P.safety, P.n_clouds, ctx->stream));
    }
    return SG_OK;
}

int drop_graph(sg_ctx* ctx) {
    if (ctx->graph) {
        cudaGraphExecDestroy(ctx->graph);
        ctx->graph = nullptr;
    }
    if (ctx->graph_timed) {
        cudaGraphExecDestroy(ctx->graph_timed);
        ctx->graph_timed = nullptr;
    }
    return SG_OK;
}

int capture_attempt(sg_ctx* ctx, Problem& P, bool timed, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    if (timed) {
        for (int k = 0; k < 12; k++)
            if (!ctx->gev[k]) CK(cudaEventCreate(&ctx->gev[k]));
        for (int k = 0; k < 2 * kStageMarks; k++)
            if (!ctx->sev[k]) CK(cudaEventCreate(&ctx->sev[k]));
    }
    CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    ctx->capture_events = timed ? 0 : -1;
    ctx->capture_stage = timed ? 0 : -1;
    // the timed graph has event nodes between its kernels: plain launches there
    const char* pdl_env = getenv("SIMGB_PDL");
    g_sg_pdl = (!timed && pdl_env && pdl_env[0] == '1') ? 1 : 0;
    int st = enqueue_attempt(ctx, P);
    g_sg_pdl = 0;
    ctx->capture_events = -1;
    if (timed) ctx->stage_pairs = ctx->capture_stage;
    ctx->capture_stage = -1;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (st != SG_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    CK(e);
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    CK(e);
    return SG_OK;
}

// The in-run force check (check.cu) after an attempt, every check_every attempts of an
// FP32c batch; its launches are not part of the attempt graph.
int maybe_check(sg_ctx* ctx, Problem& P, int attempts = 1) {
    if (!P.dchk || P.check_every <= 0 || !P.any_coulomb) return SG_OK;
    const long long before = P.attempt_count;
    P.attempt_count += attempts;
    if (P.attempt_count / P.check_every == before / P.check_every) return SG_OK;
    CK(sg_force_check(P.dc, P.n_clouds, P.ran, P.risk, P.c64, P.npad, P.coulS, P.n, P.dchk,
                      ctx->stream));
    return SG_OK;
}

// The fused small-cloud path (fused.cu) applies to FP32c Dormand-Prince batches of
// clouds of at most SG_FUSED_AUTO_IONS ions (SG_FUSED_MAX_IONS when forced) in the plain
// ion order, without a recorder,
// operations, dissociation, step log or proposer, when the device can launch a cluster
// with at most SG_FUSED_THREADS ions per CTA.
bool fused_eligible(sg_ctx* ctx, Problem& P) {
    if (!ctx->use_fused || P.precision != SG_PREC_FP32C || P.method != 5 || P.sorted ||
        P.rec_cap > 0 || !P.hops.empty() || P.n_dis > 0 || P.use_mlp || P.log_cap > 0 ||
        P.n_clouds == 0)
        return false;
    int big = 0;
    const int limit = ctx->use_fused == 2 ? SG_FUSED_MAX_IONS : SG_FUSED_AUTO_IONS;
    for (int c = 0; c < P.n_clouds; c++) {
        if (P.hc[c].n < 1 || P.hc[c].n > limit) return false;
        big = std::max(big, P.hc[c].n);
    }
    if (P.fused_cluster < 0) P.fused_cluster = sg_fused_cluster_size(P.max_npad);
    if (P.fused_cluster <= 0 || big > P.fused_cluster * SG_FUSED_THREADS) return false;
    // automatic: only while every cloud's cluster fits on the device at once; a larger
    // batch of small clouds runs faster through the batched tiled kernels (167 clouds of
    // <= 300 ions: 4.6x)
    return ctx->use_fused == 2 || (long long)P.n_clouds * P.fused_cluster <= ctx->n_sm;
}

// n attempts of every active cloud at most (a cloud stops early once done or held);
// `counted`: attempts counted towards the in-run check's interval.
int run_fused(sg_ctx* ctx, Problem& P, int n, int counted) {
    SgFusedArgs f;
    f.clouds = P.dc;
    f.ctrl = P.dctrl;
    f.y = P.y;
    f.ys = P.ys;
    f.k = P.k;
    f.coul1 = P.coul1;
    f.coul7 = P.coul7;
    f.coulS = P.coulS;
    f.kq = P.kq;
    f.qm = P.qm;
    f.c64 = P.c64;
    f.c32 = P.c32;
    f.errp = P.errp;
    f.flags = P.flags;
    f.risk = P.risk;
    f.ran = P.ran;
    f.n = P.n;
    f.npad = P.npad;
    f.n_clouds = P.n_clouds;
    f.max_attempts = n;
    TimedLaunch tl{nullptr, nullptr, 0.0, 1};
    if (ctx->timing) {
        tl.a = take_event(ctx);
        tl.b = take_event(ctx);
        CK(cudaEventRecord(tl.a, ctx->stream));
    }
    CK(sg_fused_attempts(f, P.fused_cluster, P.max_npad, ctx->stream));
    if (ctx->timing) {
        CK(cudaEventRecord(tl.b, ctx->stream));
        ctx->pending.push_back(tl);
    }
    return maybe_check(ctx, P, counted);
}

int run_attempts(sg_ctx* ctx, Problem& P, int n) {
    if (fused_eligible(ctx, P)) return run_fused(ctx, P, n, n);
    if (ctx->use_graph && ctx->timing) {
        // graph replays one at a time, reading the Coulomb event pairs after each
        if (!ctx->graph_timed) {
            int st = capture_attempt(ctx, P, true, &ctx->graph_timed);
            if (st != SG_OK) return st;
        }
        const int pairs = P.any_coulomb ? (P.method == 1 ? 1 : 6) : 0;
        const int spairs = ctx->stage_pairs;
        for (int i = 0; i < n; i++) {
            const double inter = active_interactions(P);
            CK(cudaGraphLaunch(ctx->graph_timed, ctx->stream));
            {
                int st = maybe_check(ctx, P);
                if (st != SG_OK) return st;
            }
            if (pairs) {
                CK(cudaEventSynchronize(ctx->gev[2 * pairs - 1]));
                for (int k = 0; k < pairs; k++) {
                    float ms = 0.f;
                    CK(cudaEventElapsedTime(&ms, ctx->gev[2 * k], ctx->gev[2 * k + 1]));
                    ctx->coul_ms += ms;
                    ctx->coul_launches += 1;
                    ctx->coul_inter += inter;
                }
            }
            if (spairs) {
                CK(cudaEventSynchronize(ctx->sev[2 * spairs - 1]));
                for (int k = 0; k < spairs; k++) {
                    float ms = 0.f;
                    CK(cudaEventElapsedTime(&ms, ctx->sev[2 * k], ctx->sev[2 * k + 1]));
                    ctx->stage_ms += ms;
                    ctx->stage_launches += 1;
                }
            }
        }
        return SG_OK;
    }
    if (ctx->use_graph) {
        if (!ctx->graph) {
            int st = capture_attempt(ctx, P, false, &ctx->graph);
            if (st != SG_OK) return st;
        }
        for (int i = 0; i < n; i++) {
            CK(cudaGraphLaunch(ctx->graph, ctx->stream));
            int st = maybe_check(ctx, P);
            if (st != SG_OK) return st;
        }
        return SG_OK;
    }
    for (int i = 0; i < n; i++) {
        int st = enqueue_attempt(ctx, P);
        if (st != SG_OK) return st;
        st = maybe_check(ctx, P);
        if (st != SG_OK) return st;
    }
    return SG_OK;
}

int sync_ctrl(sg_ctx* ctx, Problem& P) {
    CK(cudaMemcpyAsync(P.hctrl, P.dctrl, sizeof(SgCtrl) * P.n_clouds, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaMemcpyAsync(ctx->herr, P.flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    flush_timing(ctx);
    const int errword = *ctx->herr;
    if (errword != 0) return errword;
    return drain_records(ctx, P);
}

void fill_info(const Problem& P, sg_step_info* info) {
    if (!info) return;
    for (int c = 0; c < P.n_clouds; c++) {
        const SgCtrl& s = P.hctrl[c];
        sg_step_info& o = info[c];
        memset(&o, 0, sizeof o);
        o.t = s.t;
        o.h = s.h;
        o.h_last = s.h_last;
        o.err = s.err;
        o.errold = s.errold;
        o.steps = s.steps;
        o.rejects = s.rejects;
        o.force_evals = s.force_evals;
        o.coulomb_evals = s.coulomb_evals;
        o.status = s.status;
        o.done = s.done;
        o.reject = s.reject;
    }
}

// FP32c charge scale of each cloud from its charges (caller order): one common nonzero
// charge q gives qscale = q and normalized charges 1, so that the Coulomb kernels can skip
// the charge product; otherwise qscale = 1.
void set_charge_scale(Problem& P, const double* q) {
    for (int c = 0; c < P.n_clouds; c++) {
        SgCloud& cl = P.hc[c];
        bool uni = cl.n > 0 && q[cl.off] != 0.0;
        for (int i = cl.off + 1; uni && i < cl.off + cl.n; i++) uni = q[i] == q[cl.off];
        cl.quniform = uni ? 1 : 0;
        cl.qscale = uni ? q[cl.off] : 1.0;
    }
}

// Per-ion constants of the reference: q e/m (force.cpp:71) and the Coulomb factor
// coulomb_scale*ke*e*q*e/m written in the order of force.cpp:153.
void ion_constants(const Problem& P, const double* mass, const int* charge,
                   std::vector<double>& kq, std::vector<double>& qm, std::vector<double>& qd) {
    kq.resize(P.n);
    qm.resize(P.n);
    qd.resize(P.n);
    for (int c = 0; c < P.n_clouds; c++) {
        const SgCloud& cl = P.hc[c];
        for (int i = cl.off; i < cl.off + cl.n; i++) {
            kq[i] = cl.fp.coulomb_scale * SG_KE * SG_EL_CHARGE * charge[i] * SG_EL_CHARGE / mass[i];
            qm[i] = charge[i] * SG_EL_CHARGE / mass[i];
            qd[i] = (double)charge[i];
        }
    }
}

// Uploads positions/velocities (AoS host, caller's order) into y -- in k-d tree order for
// the sorted kernel -- brings the per-ion constants into the same order and rebuilds the
// Coulomb inputs.  The constants in the caller's order (kq0, qm0, qd0, mass0) must be on
// the device already.
// resort: a new ion order (first upload) -- the per-ion constants are gathered into it;
// otherwise they are already in place (dissociation keeps both orders current).
// sync: wait for the queued copies (the caller synchronises itself otherwise).
int upload_state(sg_ctx* ctx, Problem& P, const double* pos, const double* vel,
                 bool resort = true, bool sync = true) {
    const size_t N = (size_t)P.n;
    // the last in-attempt Coulomb sums no longer match the Coulomb inputs
    if (P.ran)
        CK(cudaMemsetAsync(P.ran, 0, sizeof(int) * (size_t)std::max(P.n_clouds, 1), ctx->stream));
    if (P.sorted && resort) {
        for (int c = 0; c < P.n_clouds; c++)
            kd_order(pos, P.hc[c].off, P.hc[c].n, P.perm.data() + P.hc[c].off);
        CK(cudaMemcpyAsync(P.dperm, P.perm.data(), sizeof(int) * N, cudaMemcpyHostToDevice,
                           ctx->stream));
    }
    CK(cudaMemcpyAsync(P.stage, pos, 3 * N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    if (vel)
        CK(cudaMemcpyAsync(P.stage + 3 * N, vel, 3 * N * sizeof(double), cudaMemcpyHostToDevice,
                           ctx->stream));
    CK(sg_aos_to_soa(P.stage, vel ? P.stage + 3 * N : nullptr, P.dperm, P.y, P.n, ctx->stream));
    if (resort) {
        CK(sg_gather(P.kq0, P.dperm, P.kq, P.n, ctx->stream));
        CK(sg_gather(P.qm0, P.dperm, P.qm, P.n, ctx->stream));
        CK(sg_gather(P.qd0, P.dperm, P.qd, P.n, ctx->stream));
        CK(sg_gather(P.mass0, P.dperm, P.mass, P.n, ctx->stream));
        CK(sg_gather_int(P.spec0, P.dperm, P.spec, P.n, ctx->stream));
        CK(sg_gather(P.pmass0, P.dperm, P.pmass, P.n, ctx->stream));
    }
    for (int c = 0; c < P.n_clouds; c++) {
        SgCloud& cl = P.hc[c];
        cl.ion0 = cl.off;
        for (int i = cl.off; i < cl.off + cl.n; i++)
            if (P.perm[i] == cl.off) {
                cl.ion0 = i;
                break;
            }
    }
    for (int c = 0; c < P.n_clouds; c++) {
        set_frame(P.hc[c], pos, P.hc[c].off);
        if (P.kfar_prior > 0.0) P.hc[c].kfar2 = (float)(P.kfar_prior * P.kfar_prior);
        double v2 = 0.0;
        if (vel)
            for (int i = P.hc[c].off; i < P.hc[c].off + P.hc[c].n; i++)
                for (int k = 0; k < 3; k++) v2 += vel[3 * (size_t)i + k] * vel[3 * (size_t)i + k];
        P.hc[c].vref = P.hc[c].n ? std::sqrt(v2 / (3.0 * P.hc[c].n)) : 0.0;
    }
    CK(cudaMemcpyAsync(P.dc, P.hc.data(), sizeof(SgCloud) * P.n_clouds, cudaMemcpyHostToDevice,
                       ctx->stream));
    SgDpArgs a = dp_args(P);
    CK(sg_coords_from_state(a, P.qd, P.n_rows, ctx->stream));
    // a new state restarts the Gear history
    if (P.method == 1) CK(sg_gear_init(a, P.dperm, P.n_rows, ctx->stream));
    // the host vectors above are read by queued copies: finish before they go away
    if (sync) CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int check_fp(const sg_field_params* fp) {
    if (!fp) return SG_BAD_ARG;
    if ((fp->flags & SG_F_PAUL) && (fp->r0 == 0.0 || fp->z0 == 0.0)) return SG_BAD_ARG;
    if ((fp->flags & SG_F_PENNING) && fp->d0 == 0.0) return SG_BAD_ARG;
    if ((fp->flags & (SG_F_QUAD | SG_F_DIPOLE)) && fp->r_el == 0.0) return SG_BAD_ARG;
    return SG_OK;
}

// Prepares `solo` for a stand-alone call on n ions.
int solo_prepare(sg_ctx* ctx, int n, int precision, const sg_field_params& fp) {
    Problem& P = ctx->solo;
    const bool same = P.n_clouds == 1 && P.n == n && P.precision == precision &&
                      P.variant == auto_variant(std::vector<int>(1, n), ctx->c32_variant) &&
                      ((P.hc[0].fp.flags & SG_F_COULOMB) == (fp.flags & SG_F_COULOMB));
    if (!same) {
        free_problem(P);
        P.n_clouds = 1;
        P.counts.assign(1, n);
        P.precision = precision;
        P.variant = auto_variant(P.counts, ctx->c32_variant);
        P.hc.assign(1, SgCloud());
        P.hc[0].fp = fp;
        plan(P, ctx->n_sm);
        int st = alloc_problem(ctx, P);
        if (st != SG_OK) {
            free_problem(P);
            return st;
        }
    }
    P.hc[0].fp = fp;
    return SG_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

int sg_version(void) { return 100; }

const char* sg_status_string(int s) {
    switch (s) {
        case SG_OK: return "ok";
        case SG_BAD_ARG: return "bad argument";
        case SG_CUDA_ERR: return "CUDA error";
        case SG_H_UNDERFLOW: return "stepsize underflow created";
        case SG_NONFINITE: return "non-finite error norm";
        case SG_TIMEOUT: return "device wait timed out";
        case SG_NO_DEVICE: return "no CUDA device";
        case SG_TOO_MANY_REJECTS: return "too many rejected attempts";
        case SG_NOT_READY: return "state not uploaded";
        case SG_TOO_LARGE: return "size exceeds the fixed capacity";
        case SG_IO_ERR: return "file could not be read or written";
        default: return "unknown status";
    }
}

int sg_create(int device, sg_ctx** out) {
    if (!out) return SG_BAD_ARG;
    *out = nullptr;
    int nd = 0;
    if (cudaGetDeviceCount(&nd) != cudaSuccess || nd <= 0) return SG_NO_DEVICE;
    if (device < 0 || device >= nd) return SG_BAD_ARG;
    sg_ctx* ctx = new sg_ctx();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) {
        delete ctx;
        return SG_NO_DEVICE;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) ctx->n_sm = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&ctx->t0) != cudaSuccess || cudaEventCreate(&ctx->t1) != cudaSuccess ||
        cudaMallocHost((void**)&ctx->herr, sizeof(int)) != cudaSuccess) {
        delete ctx;
        return SG_CUDA_ERR;
    }
    *out = ctx;
    return SG_OK;
}

int sg_destroy(sg_ctx* ctx) {
    if (!ctx) return SG_BAD_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    flush_timing(ctx);
    drop_graph(ctx);
    free_problem(ctx->batch);
    free_problem(ctx->solo);
    for (cudaEvent_t e : ctx->free_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->gev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->sev)
        if (e) cudaEventDestroy(e);
    cudaEventDestroy(ctx->t0);
    cudaEventDestroy(ctx->t1);
    cudaFree(ctx->probe_sink);
    float* mf[] = {ctx->mlp_wm, ctx->mlp_m1, ctx->mlp_m2, ctx->mlp_grad, ctx->mlp_gpart,
                   ctx->mlp_lpart, ctx->mlp_loss, ctx->mlp_X, ctx->mlp_Y, ctx->mlp_out};
    for (float* f : mf) cudaFree(f);
    cudaFree(ctx->mlp_idx);
    cudaFree(ctx->mlp_wbf);
    cudaFree(ctx->cb_xj);
    cudaFree(ctx->cb_mj);
    cudaFree(ctx->cb_xi);
    cudaFree(ctx->cb_ai);
    if (ctx->cb_host) cudaFreeHost(ctx->cb_host);
    cudaFreeHost(ctx->herr);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SG_OK;
}

int sg_last_cuda_error(sg_ctx* ctx) { return ctx ? ctx->last_err : 0; }

int sg_sync(sg_ctx* ctx) {
    if (!ctx) return SG_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    flush_timing(ctx);
    return SG_OK;
}

int sg_coulomb_accel(sg_ctx* ctx, int precision, int n, const double* pos, const double* q,
                     const double* kq, double* acc) {
    if (!ctx || n < 0 || (n > 0 && (!pos || !q || !kq || !acc))) return SG_BAD_ARG;
    if (precision != SG_PREC_FP64 && precision != SG_PREC_FP32C) return SG_BAD_ARG;
    if (n == 0) return SG_OK;
    CK(cudaSetDevice(ctx->device));
    sg_field_params fp;
    memset(&fp, 0, sizeof fp);
    fp.flags = SG_F_COULOMB;
    fp.coulomb_scale = 1.0;
    int st = solo_prepare(ctx, n, precision, fp);
    if (st != SG_OK) return st;
    Problem& P = ctx->solo;
    CK(cudaMemcpyAsync(P.qd0, q, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    set_charge_scale(P, q);
    CK(cudaMemcpyAsync(P.kq0, kq, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    st = upload_state(ctx, P, pos, nullptr);
    if (st != SG_OK) return st;
    st = launch_coulomb(ctx, P, false, (double)n * (n - 1), P.coulS);
    if (st != SG_OK) return st;
    SgDpArgs a = dp_args(P);
    CK(sg_force_finish(a, 0.0, 0, P.dperm, P.stage, P.n_rows, ctx->stream));
    CK(cudaMemcpyAsync(acc, P.stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
    int errword = 0;
    CK(cudaMemcpyAsync(&errword, P.flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    flush_timing(ctx);
    return errword ? errword : SG_OK;
}

int sg_force(sg_ctx* ctx, int precision, int n, const double* pos, const double* vel,
             const double* mass, const int* charge, double t, const sg_field_params* fp,
             double* acc) {
    if (!ctx || n < 0 || (n > 0 && (!pos || !vel || !mass || !charge || !acc))) return SG_BAD_ARG;
    if (precision != SG_PREC_FP64 && precision != SG_PREC_FP32C) return SG_BAD_ARG;
    if (check_fp(fp) != SG_OK) return SG_BAD_ARG;
    if (n == 0) return SG_OK;
    CK(cudaSetDevice(ctx->device));
    int st = solo_prepare(ctx, n, precision, *fp);
    if (st != SG_OK) return st;
    Problem& P = ctx->solo;
    std::vector<double> kq, qm, qd;
    ion_constants(P, mass, charge, kq, qm, qd);
    set_charge_scale(P, qd.data());
    CK(cudaMemcpyAsync(P.qd0, qd.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(P.kq0, kq.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(P.qm0, qm.data(), sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(P.mass0, mass, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    st = upload_state(ctx, P, pos, vel);
    if (st != SG_OK) return st;
    if (fp->flags & SG_F_COULOMB) {
        st = launch_coulomb(ctx, P, false, (double)n * (n - 1), P.coulS);
        if (st != SG_OK) return st;
    }
    SgDpArgs a = dp_args(P);
    CK(sg_force_finish(a, t, 1, P.dperm, P.stage, P.n_rows, ctx->stream));
    CK(cudaMemcpyAsync(acc, P.stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
    int errword = 0;
    CK(cudaMemcpyAsync(&errword, P.flags, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    flush_timing(ctx);
    return errword ? errword : SG_OK;
}

int sg_batch_create(sg_ctx* ctx, int n_clouds, const int* counts, const sg_field_params* fp,
                    const sg_ode_params* op, int precision) {
    if (!ctx || n_clouds <= 0 || !counts || !fp || !op) return SG_BAD_ARG;
    if (precision != SG_PREC_FP64 && precision != SG_PREC_FP32C) return SG_BAD_ARG;
    long long total = 0;
    for (int c = 0; c < n_clouds; c++) {
        if (counts[c] <= 0 || check_fp(&fp[c]) != SG_OK) return SG_BAD_ARG;
        if (!(op[c].rtol >= 0.0) || !(op[c].atol >= 0.0) || !(op[c].h0 > 0.0)) return SG_BAD_ARG;
        const int m = op[c].method == 0 ? 5 : op[c].method;
        const int m0 = op[0].method == 0 ? 5 : op[0].method;
        if ((m != 5 && m != 4 && m != 1) || m != m0) return SG_BAD_ARG;
        total += counts[c];
    }
    if (total > (1ll << 30)) return SG_BAD_ARG;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    flush_timing(ctx);
    drop_graph(ctx);
    free_problem(ctx->batch);
    Problem& P = ctx->batch;
    P.n_clouds = n_clouds;
    P.counts.assign(counts, counts + n_clouds);
    P.precision = precision;
    P.variant = auto_variant(P.counts, ctx->c32_variant);
    P.method = op[0].method == 0 ? 5 : op[0].method;
    P.hc.assign(n_clouds, SgCloud());
    for (int c = 0; c < n_clouds; c++) P.hc[c].fp = fp[c];
    P.fp0.assign(fp, fp + n_clouds);
    plan(P, ctx->n_sm);
    P.hctrl0.assign(n_clouds, SgCtrl());
    for (int c = 0; c < n_clouds; c++) {
        SgCtrl& s = P.hctrl0[c];
        memset(&s, 0, sizeof s);
        s.t = op[c].t0;
        s.h = op[c].h0;
        s.hnext = op[c].h0;
        s.errold = 1.0e-4;  // Init_ode, bin/ode.cpp:540
        s.t_end = op[c].t_end;
        s.rtol = op[c].rtol;
        s.atol = op[c].atol;
        s.adaptive = op[c].adaptive;
        s.max_rejects = op[c].max_rejects;
        s.beta = op[c].beta;
        s.method = P.method;
        {
            // Init_ode's step powers (bin/ode.cpp:548-552); the reference is C++98, where
            // pow(double, int) multiplies out: h^3 = h^2 h, h^4 = h^2 h^2, h^5 = h^3 h^2
            const double h1 = op[c].h0, h2 = h1 * h1, h3 = h2 * h1;
            s.hf[0] = h1 * h1 / 2.;
            s.hf[1] = h3 / 6.;
            s.hf[2] = h2 * h2 / 24.;
            s.hf[3] = h3 * h2 / 120.;
        }
        s.err = 0.0;
        s.status = SG_OK;
        s.done = (s.t >= s.t_end) ? 1 : 0;
    }
    int st = alloc_problem(ctx, P);
    if (st != SG_OK) {
        free_problem(P);
        return st;
    }
    memcpy(P.hctrl, P.hctrl0.data(), sizeof(SgCtrl) * n_clouds);
    P.rec_host.assign(n_clouds, std::vector<double>());
    P.hspec0.assign(P.n, 0);
    P.hmass0.assign(P.n, 0.0);
    return SG_OK;
}

int sg_batch_upload(sg_ctx* ctx, const double* pos, const double* vel, const double* mass,
                    const int* charge) {
    if (!ctx || !pos || !vel || !mass || !charge) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    for (int i = 0; i < P.n; i++)
        if (!(mass[i] > 0.0)) return SG_BAD_ARG;
    CK(cudaSetDevice(ctx->device));
    std::vector<double> kq, qm, qd;
    ion_constants(P, mass, charge, kq, qm, qd);
    set_charge_scale(P, qd.data());
    const size_t N = (size_t)P.n;
    CK(cudaMemcpyAsync(P.kq0, kq.data(), N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(P.qm0, qm.data(), N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(P.qd0, qd.data(), N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(P.mass0, mass, N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    P.hmass0.assign(mass, mass + N);
    CK(cudaMemcpyAsync(P.pmass0, mass, N * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(P.spec0, P.hspec0.data(), N * sizeof(int), cudaMemcpyHostToDevice,
                       ctx->stream));
    for (auto& r : P.rec_host) r.clear();  // records of the previous state
    memcpy(P.hctrl, P.hctrl0.data(), sizeof(SgCtrl) * P.n_clouds);
    // the operation sequence restarts from the caller's field parameters
    for (int c = 0; c < P.n_clouds; c++) {
        P.hc[c].fp = P.fp0[c];
        if (!P.hops.empty()) sg_start_ops(P.hctrl[c], P.hc[c].fp, P.hops.data(), 0);
    }
    {
        int st0 = dissociation_tables(ctx, P);
        if (st0 != SG_OK) return st0;
    }
    CK(cudaMemcpyAsync(P.dctrl, P.hctrl, sizeof(SgCtrl) * P.n_clouds, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaMemsetAsync(P.flags, 0, 4 * sizeof(int), ctx->stream));
    int st = upload_state(ctx, P, pos, vel);
    if (st != SG_OK) return st;
    // a dissociation at the very start of the sequence
    if (P.n_dis > 0)
        CK(sg_dissociate(rec_args(P), P.pmass, P.spec0, P.pmass0, P.n_rows, ctx->stream));
    // stage-1 Coulomb sum of the initial state
    st = launch_coulomb(ctx, P, true, active_interactions(P), P.coul1);
    if (st != SG_OK) return st;
    st = proposer_reset(ctx, P);
    if (st != SG_OK) return st;
    CK(cudaStreamSynchronize(ctx->stream));
    flush_timing(ctx);
    P.uploaded = true;
    drop_graph(ctx);  // frames changed: the captured kernels read them from memory, but
                      // re-capturing keeps the graph tied to the current buffers
    return SG_OK;
}

int sg_batch_set_state(sg_ctx* ctx, const double* pos, const double* vel) {
    if (!ctx || !pos || !vel) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (!P.uploaded) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    // field parameters as the device has them now (only an operation sequence moves them)
    if (!P.hops.empty()) CK(pull_clouds(ctx, P));
    // a continuing run keeps its ion order: the tile bounds are recomputed from the new
    // positions at every stage, so an older k-d order costs some far pairs, never accuracy
    int st = upload_state(ctx, P, pos, vel, false, false);
    if (st != SG_OK) return st;
    st = launch_coulomb(ctx, P, true, active_interactions(P), P.coul1);
    if (st != SG_OK) return st;
    st = proposer_reset(ctx, P);
    if (st != SG_OK) return st;
    CK(cudaStreamSynchronize(ctx->stream));
    flush_timing(ctx);
    return SG_OK;
}

int sg_batch_download(sg_ctx* ctx, double* pos, double* vel) {
    if (!ctx || !pos || !vel) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (!P.uploaded) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    const size_t N = (size_t)P.n;
    CK(sg_soa_to_aos(P.y, P.dperm, P.stage, P.stage + 3 * N, P.n, ctx->stream));
    CK(cudaMemcpyAsync(pos, P.stage, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(vel, P.stage + 3 * N, 3 * N * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_batch_attempts(sg_ctx* ctx, int n_attempts) {
    if (!ctx || n_attempts < 0) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (!P.uploaded) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    return run_attempts(ctx, P, n_attempts);
}

int sg_dp45_step(sg_ctx* ctx, sg_step_info* info) {
    if (!ctx) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (!P.uploaded) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    // hold-on-accept on (any nonzero word) without a host-to-device copy
    CK(cudaMemsetAsync(P.flags + 1, 1, sizeof(int), ctx->stream));
    int st = SG_OK;
    // every cloud that is active now takes exactly one accepted step (or fails); the
    // fused path loops over a cloud's attempts inside one launch until it holds
    const bool fused = fused_eligible(ctx, P);
    for (long long guard = 0; guard < (1ll << 40); guard++) {
        st = fused ? run_fused(ctx, P, 64, 1) : run_attempts(ctx, P, 1);
        if (st != SG_OK) break;
        st = sync_ctrl(ctx, P);
        if (st != SG_OK) break;
        bool all = true;
        for (int c = 0; c < P.n_clouds; c++) {
            const SgCtrl& s = P.hctrl[c];
            if (!(s.done || s.hold || s.status != SG_OK)) all = false;
        }
        if (all) break;
    }
    CK(cudaMemsetAsync(P.flags + 1, 0, sizeof(int), ctx->stream));
    CK(sg_clear_hold(P.dctrl, P.n_clouds, ctx->stream));
    if (st == SG_OK) {
        // the host copy is current from the last sync: clear its hold bit the same way
        // instead of reading the control blocks back once more
        for (int c = 0; c < P.n_clouds; c++) P.hctrl[c].hold &= ~1;
    } else {
        int st2 = sync_ctrl(ctx, P);
        (void)st2;
    }
    fill_info(P, info);
    if (st != SG_OK) return st;
    for (int c = 0; c < P.n_clouds; c++)
        if (P.hctrl[c].status != SG_OK) return P.hctrl[c].status;
    return SG_OK;
}

int sg_batch_run(sg_ctx* ctx, int64_t max_attempts, sg_step_info* info) {
    if (!ctx || max_attempts < 0) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (!P.uploaded) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    int st = sync_ctrl(ctx, P);
    int64_t done_attempts = 0;
    int chunk = 1;
    while (st == SG_OK && done_attempts < max_attempts) {
        bool all = true;
        for (int c = 0; c < P.n_clouds; c++)
            if (!P.hctrl[c].done && P.hctrl[c].status == SG_OK) all = false;
        if (all) break;
        const int n = (int)std::min<int64_t>(chunk, max_attempts - done_attempts);
        st = run_attempts(ctx, P, n);
        if (st != SG_OK) break;
        done_attempts += n;
        st = sync_ctrl(ctx, P);
        chunk = std::min(chunk * 2, 64);
    }
    fill_info(P, info);
    return st;
}


// ---- recorder: device-side observables and the reference's text output ------------
int sg_batch_set_recorder(sg_ctx* ctx, double print_interval, int stride, int capacity,
                          const int* species, int n_species) {
    if (!ctx || stride < 1 || capacity < 0 || n_species < 1 || n_species > SG_MAX_SPECIES ||
        !(print_interval >= 0.0))
        return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    if (species)
        for (int i = 0; i < P.n; i++)
            if (species[i] < 0 || species[i] >= n_species) return SG_BAD_ARG;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    drop_graph(ctx);  // the attempt sequence gains or loses the record kernels
    cudaFree(P.ring);
    P.ring = nullptr;
    P.rec_cap = capacity;
    P.rec_stride = stride;
    P.n_species = n_species;
    P.print_interval = print_interval;
    if (species)
        P.hspec0.assign(species, species + P.n);
    else
        P.hspec0.assign(P.n, 0);
    long long off = 0;
    for (int c = 0; c < P.n_clouds; c++) {
        SgCloud& cl = P.hc[c];
        cl.nsel = (cl.n + stride - 1) / stride;
        cl.rec_len = 1 + SG_STAT_LEN * n_species + SG_ION_LEN * cl.nsel;
        cl.rec_off = off;
        off += (long long)capacity * cl.rec_len;
    }
    if (capacity > 0) CK(dalloc(&P.ring, (size_t)off));
    {
        // keep the device's field parameters (a ramp may have moved them)
        std::vector<SgCloud> cur(P.n_clouds);
        CK(cudaMemcpy(cur.data(), P.dc, sizeof(SgCloud) * P.n_clouds, cudaMemcpyDeviceToHost));
        for (int c = 0; c < P.n_clouds; c++) P.hc[c].fp = cur[c].fp;
    }
    CK(cudaMemcpyAsync(P.spec0, P.hspec0.data(), sizeof(int) * P.n, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(sg_gather_int(P.spec0, P.dperm, P.spec, P.n, ctx->stream));
    CK(cudaMemcpyAsync(P.dc, P.hc.data(), sizeof(SgCloud) * P.n_clouds, cudaMemcpyHostToDevice,
                       ctx->stream));
    P.rec_host.assign(P.n_clouds, std::vector<double>());
    // the print clock starts now: at the initial time before an upload, else at t
    CK(cudaMemcpyAsync(P.hctrl, P.dctrl, sizeof(SgCtrl) * P.n_clouds, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < P.n_clouds; c++) {
        for (SgCtrl* s : {&P.hctrl0[c], &P.hctrl[c]}) {
            s->print_interval = print_interval;
            s->t_print0 = s->t;
            s->n_print = 0;
            s->rec_count = 0;
            s->rec_drained = 0;
            s->rec_cap = capacity;
            s->print_due = 0;
            s->hold &= ~2;
        }
        P.hctrl0[c].t_print0 = P.hctrl0[c].t;
    }
    if (!P.uploaded) memcpy(P.hctrl, P.hctrl0.data(), sizeof(SgCtrl) * P.n_clouds);
    CK(cudaMemcpyAsync(P.dctrl, P.hctrl, sizeof(SgCtrl) * P.n_clouds, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_batch_record_now(sg_ctx* ctx) {
    if (!ctx) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (!P.uploaded) return SG_NOT_READY;
    if (P.rec_cap <= 0) return SG_BAD_ARG;
    CK(cudaSetDevice(ctx->device));
    int st = sync_ctrl(ctx, P);  // drains: the rings have room
    if (st != SG_OK) return st;
    CK(sg_record_now(P.dctrl, P.n_clouds, ctx->stream));
    CK(sg_record(rec_args(P), P.n_rows, P.n_clouds, ctx->stream));
    return sync_ctrl(ctx, P);
}

int sg_batch_records(sg_ctx* ctx, int cloud, int64_t* n_records, int* record_len,
                     int* n_kept) {
    if (!ctx) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    if (cloud < 0 || cloud >= P.n_clouds) return SG_BAD_ARG;
    const SgCloud& cl = P.hc[cloud];
    const int len = P.rec_cap > 0 ? cl.rec_len : 0;
    if (n_records) *n_records = len ? (int64_t)(P.rec_host[cloud].size() / len) : 0;
    if (record_len) *record_len = len;
    if (n_kept) *n_kept = P.rec_cap > 0 ? cl.nsel : 0;
    return SG_OK;
}

int sg_batch_read_records(sg_ctx* ctx, int cloud, int64_t max_records, double* out,
                          int64_t* n_read) {
    if (!ctx || max_records < 0 || (max_records > 0 && !out)) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    if (cloud < 0 || cloud >= P.n_clouds || P.rec_cap <= 0) return SG_BAD_ARG;
    const size_t len = (size_t)P.hc[cloud].rec_len;
    std::vector<double>& src = P.rec_host[cloud];
    const int64_t k = std::min<int64_t>(max_records, (int64_t)(src.size() / len));
    if (k > 0) {
        memcpy(out, src.data(), sizeof(double) * len * (size_t)k);
        src.erase(src.begin(), src.begin() + (ptrdiff_t)(len * (size_t)k));
    }
    if (n_read) *n_read = k;
    return SG_OK;
}

namespace {
// File header of the reference's output files (bin/ioncloud.cpp:227-235, 246-253).
void write_header(FILE* f, const char* columns) {
    time_t now = time(nullptr);
    fprintf(f, "#Simulation started: %s", ctime(&now));
    fputs("#------------------------------------------------------------------------------#\n", f);
    fputs("#                          JILA EDM Paul Trap Simulation                       #\n", f);
    fputs("#      Dormand-Prince Runga-Kutta with Proportional Integrating controller     #\n", f);
    fputs("#------------------------------------------------------------------------------#\n", f);
    fputs(columns, f);
    fputs("#*******************************************************************************\n", f);
}

FILE* open_append(const std::string& name, const char* columns) {
    FILE* f = fopen(name.c_str(), "a");
    if (f && ftell(f) == 0) write_header(f, columns);
    return f;
}
}  // namespace

// PrintParticles / PrintCloud lines (bin/ioncloud.cpp:85-183) for the drained records of
// one cloud, appended to <prefix>_pAll.txt and <prefix>_cloud<s>.txt; the records are
// consumed.  Scientific notation with 6 digits, as the reference's streams are set up.
int sg_batch_write_text(sg_ctx* ctx, int cloud, const char* prefix, const char* const* names,
                        int n_names) {
    if (!ctx || !prefix || !names) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    if (cloud < 0 || cloud >= P.n_clouds || P.rec_cap <= 0 || n_names < P.n_species)
        return SG_BAD_ARG;
    const SgCloud& cl = P.hc[cloud];
    const size_t len = (size_t)cl.rec_len;
    std::vector<double>& recs = P.rec_host[cloud];
    const size_t nrec = recs.size() / len;
    FILE* fa = open_append(std::string(prefix) + "_pAll.txt",
                           "#index \t mass \t t (ms) \t x y z (mm) vx vy vz (m/s) \t Energy(eV)\n");
    if (!fa) return SG_BAD_ARG;
    std::vector<FILE*> fc(P.n_species, nullptr);
    for (int s = 0; s < P.n_species; s++) {
        fc[s] = open_append(std::string(prefix) + "_cloud" + std::to_string(s) + ".txt",
                            "#index \t type \t #particules \t t (ms) \t x0 y0 z0 (mm) sx sy sz (m/s) \t Energy(eV)\n");
        if (!fc[s]) {
            fclose(fa);
            for (FILE* f : fc)
                if (f) fclose(f);
            return SG_BAD_ARG;
        }
    }
    for (size_t r = 0; r < nrec; r++) {
        const double* rec = recs.data() + r * len;
        const double t = rec[0];
        const double* ions = rec + 1 + SG_STAT_LEN * P.n_species;
        for (int j = 0; j < cl.nsel; j++) {
            const int loc = j * P.rec_stride;
            const double* y = ions + SG_ION_LEN * j;
            const int sp = (int)y[7];
            fprintf(fa, "%d %s %e %e %e %e %e %e %e %e\n", loc, names[sp], t * 1000.0,
                    y[0] * 1000.0, y[1] * 1000.0, y[2] * 1000.0, y[3], y[4], y[5], y[6]);
        }
        for (int s = 0; s < P.n_species; s++) {
            const double* o = rec + 1 + SG_STAT_LEN * s;
            fprintf(fc[s], "%d %s %d %e %e %e %e %e %e %e %e\n", s, names[s], (int)o[8], t * 1e3,
                    1000.0 * o[0], 1000.0 * o[1], 1000.0 * o[2], 1000.0 * o[3], 1000.0 * o[4],
                    1000.0 * o[5], o[6]);
        }
    }
    fclose(fa);
    for (FILE* f : fc) fclose(f);
    recs.clear();
    return SG_OK;
}


// ---- operation sequence -----------------------------------------------------------
int sg_batch_set_operations(sg_ctx* ctx, const sg_operation* ops, int n_ops) {
    if (!ctx || n_ops < 0 || n_ops > 64 || (n_ops > 0 && !ops)) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    std::vector<SgOp> h(n_ops);
    int d = 0;
    for (int k = 0; k < n_ops; k++) {
        const sg_operation& o = ops[k];
        if (o.kind < SG_OP_NORMAL || o.kind > SG_OP_DISSOCIATION) return SG_BAD_ARG;
        if (!(o.duration >= 0.0) || !(o.print_time >= 0.0)) return SG_BAD_ARG;
        // ode_timestep sets the step to print_time: it must be a step
        if (o.timestep != 0.0 && !(o.print_time > 0.0)) return SG_BAD_ARG;
        if (o.kind == SG_OP_DISSOCIATION &&
            (o.reactant < 0 || o.reactant >= SG_MAX_SPECIES || o.product < 0 ||
             o.product >= SG_MAX_SPECIES || !(o.product_mass > 0.0)))
            return SG_BAD_ARG;
        SgOp& q = h[k];
        memset(&q, 0, sizeof q);
        q.kind = o.kind;
        q.print_after = o.print_after != 0;
        q.duration = o.kind == SG_OP_DISSOCIATION ? 0.0 : o.duration;
        q.print_time = o.print_time;
        q.timestep = o.timestep;
        q.new_vrf = o.new_vrf;
        q.new_vdc = o.new_vdc;
        q.e_kick = o.e_kick;
        q.reactant = o.reactant;
        q.product = o.product;
        q.fraction = o.fraction;
        q.product_mass = o.product_mass;
        q.dis_index = o.kind == SG_OP_DISSOCIATION ? d++ : -1;
    }
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    drop_graph(ctx);
    cudaFree(P.dops);
    P.dops = nullptr;
    P.hops = h;
    if (n_ops > 0) {
        CK(dalloc(&P.dops, (size_t)n_ops));
        CK(cudaMemcpy(P.dops, h.data(), sizeof(SgOp) * n_ops, cudaMemcpyHostToDevice));
    }
    for (int c = 0; c < P.n_clouds; c++) {
        const int bits = P.fp0[c].flags & (SG_F_PAUL | SG_F_PENNING);
        P.hctrl0[c].n_ops = n_ops;
        P.hctrl0[c].trap_bits = bits;
        P.hctrl0[c].op_index = 0;
        P.hctrl0[c].dis_due = 0;
    }
    if (!P.uploaded) return dissociation_tables(ctx, P);
    // start the sequence now, from the caller's field parameters, at each cloud's time
    int st = sync_ctrl(ctx, P);
    if (st != SG_OK) return st;
    for (int c = 0; c < P.n_clouds; c++) {
        SgCtrl& cs = P.hctrl[c];
        cs.n_ops = n_ops;
        cs.trap_bits = P.hctrl0[c].trap_bits;
        cs.dis_due = 0;
        P.hc[c].fp = P.fp0[c];
        if (n_ops > 0 && cs.status == SG_OK) {
            cs.done = 0;
            sg_start_ops(cs, P.hc[c].fp, P.hops.data(), 0);
        }
    }
    st = dissociation_tables(ctx, P);
    if (st != SG_OK) return st;
    {
        std::vector<SgCloud> cur(P.n_clouds);
        CK(cudaMemcpy(cur.data(), P.dc, sizeof(SgCloud) * P.n_clouds, cudaMemcpyDeviceToHost));
        for (int c = 0; c < P.n_clouds; c++) cur[c].fp = P.hc[c].fp;
        CK(cudaMemcpy(P.dc, cur.data(), sizeof(SgCloud) * P.n_clouds, cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(P.dctrl, P.hctrl, sizeof(SgCtrl) * P.n_clouds, cudaMemcpyHostToDevice));
    if (P.n_dis > 0)
        CK(sg_dissociate(rec_args(P), P.pmass, P.spec0, P.pmass0, P.n_rows, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_batch_operation_index(sg_ctx* ctx, int* index) {
    if (!ctx || !index) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    int st = sync_ctrl(ctx, P);
    if (st != SG_OK) return st;
    for (int c = 0; c < P.n_clouds; c++) index[c] = P.hctrl[c].op_index;
    return SG_OK;
}

int sg_batch_info(sg_ctx* ctx, sg_step_info* info) {
    if (!ctx || !info) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    int st = sync_ctrl(ctx, P);
    fill_info(P, info);
    return st;
}

int sg_batch_set_field(sg_ctx* ctx, int cloud, const sg_field_params* fp) {
    if (!ctx || check_fp(fp) != SG_OK) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (cloud < 0 || cloud >= P.n_clouds) return SG_BAD_ARG;
    if ((fp->flags & SG_F_COULOMB) != (P.hc[cloud].fp.flags & SG_F_COULOMB)) return SG_BAD_ARG;
    CK(cudaSetDevice(ctx->device));
    P.hc[cloud].fp = *fp;
    P.fp0[cloud] = *fp;
    CK(cudaMemcpyAsync(&P.dc[cloud].fp, fp, sizeof(sg_field_params), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_batch_set_t_end(sg_ctx* ctx, int cloud, double t_end) {
    if (!ctx) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (cloud < 0 || cloud >= P.n_clouds) return SG_BAD_ARG;
    CK(cudaSetDevice(ctx->device));
    int st = sync_ctrl(ctx, P);
    if (st != SG_OK) return st;
    SgCtrl s = P.hctrl[cloud];
    s.t_end = t_end;
    if (s.status == SG_OK) s.done = (s.t >= t_end) ? 1 : 0;
    P.hctrl[cloud] = s;
    CK(cudaMemcpyAsync(&P.dctrl[cloud], &P.hctrl[cloud], sizeof(SgCtrl), cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_set_kernel_timing(sg_ctx* ctx, int on) {
    if (!ctx) return SG_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    flush_timing(ctx);
    ctx->timing = on != 0;
    ctx->coul_ms = 0.0;
    ctx->coul_inter = 0.0;
    ctx->coul_launches = 0;
    ctx->stage_ms = 0.0;
    ctx->stage_launches = 0;
    ctx->fused_ms = 0.0;
    ctx->fused_launches = 0;
    return SG_OK;
}

int sg_stage_timing(sg_ctx* ctx, double* ms, int64_t* launches) {
    if (!ctx) return SG_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    if (ms) *ms = ctx->stage_ms;
    if (launches) *launches = ctx->stage_launches;
    return SG_OK;
}

int sg_kernel_timing(sg_ctx* ctx, double* coulomb_ms, int64_t* launches, double* inter) {
    if (!ctx) return SG_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    flush_timing(ctx);
    if (coulomb_ms) *coulomb_ms = ctx->coul_ms;
    if (launches) *launches = ctx->coul_launches;
    if (inter) *inter = ctx->coul_inter;
    return SG_OK;
}

int sg_fixup_count(sg_ctx* ctx, int64_t* count) {
    if (!ctx || !count) return SG_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    *count = 0;
    Problem* ps[2] = {&ctx->batch, &ctx->solo};
    for (Problem* P : ps) {
        if (!P->flags) continue;
        int v = 0;
        CK(cudaMemcpy(&v, P->flags + 2, sizeof(int), cudaMemcpyDeviceToHost));
        CK(cudaMemset(P->flags + 2, 0, sizeof(int)));
        *count += v;
    }
    return SG_OK;
}

int sg_set_coulomb_variant(sg_ctx* ctx, int variant) {
    if (!ctx || variant < -1 || variant >= SG_C32_VARIANTS) return SG_BAD_ARG;
    ctx->c32_variant = variant;
    return SG_OK;
}

int sg_batch_variant(sg_ctx* ctx, int* variant) {
    if (!ctx || !variant) return SG_BAD_ARG;
    if (ctx->batch.n_clouds == 0) return SG_NOT_READY;
    *variant = ctx->batch.precision == SG_PREC_FP32C ? ctx->batch.variant : 0;
    return SG_OK;
}

int sg_set_fused(sg_ctx* ctx, int on) {
    if (!ctx) return SG_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    if (on < 0 || on > 2) return SG_BAD_ARG;
    ctx->use_fused = on;
    return SG_OK;
}

int sg_fused_timing(sg_ctx* ctx, double* ms, int64_t* launches) {
    if (!ctx) return SG_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    flush_timing(ctx);
    if (ms) *ms = ctx->fused_ms;
    if (launches) *launches = ctx->fused_launches;
    return SG_OK;
}

int sg_batch_fused(sg_ctx* ctx, int* cluster) {
    if (!ctx || !cluster) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    *cluster = fused_eligible(ctx, P) ? P.fused_cluster : 0;
    return SG_OK;
}

int sg_set_use_graph(sg_ctx* ctx, int on) {
    if (!ctx) return SG_BAD_ARG;
    CK(cudaStreamSynchronize(ctx->stream));
    drop_graph(ctx);
    ctx->use_graph = on != 0;
    return SG_OK;
}

int sg_timer_start(sg_ctx* ctx) {
    if (!ctx) return SG_BAD_ARG;
    CK(cudaEventRecord(ctx->t0, ctx->stream));
    return SG_OK;
}

int sg_timer_stop(sg_ctx* ctx, double* ms) {
    if (!ctx || !ms) return SG_BAD_ARG;
    CK(cudaEventRecord(ctx->t1, ctx->stream));
    CK(cudaEventSynchronize(ctx->t1));
    float f = 0.f;
    CK(cudaEventElapsedTime(&f, ctx->t0, ctx->t1));
    *ms = f;
    return SG_OK;
}

int sg_batch_moments(sg_ctx* ctx, double* out) {
    if (!ctx || !out) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (!P.uploaded) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    SgDpArgs a = dp_args(P);
    CK(sg_moments(a, P.mass, P.mom, P.n_rows, ctx->stream));
    std::vector<double> h((size_t)P.n_rows * 11);
    CK(cudaMemcpyAsync(h.data(), P.mom, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < P.n_clouds; c++) {
        const SgCloud& cl = P.hc[c];
        double s[11] = {0};
        for (int b = 0; b < cl.nrb; b++)
            for (int q = 0; q < 11; q++) s[q] += h[(size_t)(cl.rb0 + b) * 11 + q];
        double* o = out + 12 * (size_t)c;
        const double n = cl.n;
        for (int ax = 0; ax < 3; ax++) {
            const double m = s[ax] / n;
            o[ax] = m;
            const double var = s[3 + ax] / n - m * m;
            o[3 + ax] = var > 0 ? std::sqrt(var) : 0.0;
            o[6 + ax] = s[6 + ax] / n;
        }
        // IonCloud::Temperature (bin/ioncloud.cpp:316-335)
        o[9] = s[9] * (0.5 / n) * (2.0 / (3.0 * SG_KB));
        o[10] = s[10] * (0.5 / n) * (2.0 / (3.0 * SG_KB));
        o[11] = n;
    }
    return SG_OK;
}

int sg_probe_peaks(sg_ctx* ctx, double* fp32, double* fp32x2, double* fp64) {
    if (!ctx) return SG_BAD_ARG;
    CK(cudaSetDevice(ctx->device));
    const int blocks = ctx->n_sm * 8, threads = 256;
    if (!ctx->probe_sink) CK(dalloc(&ctx->probe_sink, (size_t)blocks * threads));
    double* outs[3] = {fp32, fp32x2, fp64};
    for (int w = 0; w < 3; w++) {
        if (!outs[w]) continue;
        CK(sg_probe_launch(w, blocks, threads, ctx->probe_sink, ctx->stream));  // warm-up
        double best = 0.0;
        for (int rep = 0; rep < 3; rep++) {
            CK(cudaEventRecord(ctx->t0, ctx->stream));
            CK(sg_probe_launch(w, blocks, threads, ctx->probe_sink, ctx->stream));
            CK(cudaEventRecord(ctx->t1, ctx->stream));
            CK(cudaEventSynchronize(ctx->t1));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ctx->t0, ctx->t1));
            const double flops = 2.0 * 8.0 * sg_probe_iters(w) * (double)blocks * threads;
            best = std::max(best, flops / (ms * 1e-3) / 1e9);
        }
        *outs[w] = best;
    }
    return SG_OK;
}

}  // extern "C"


// ---- learned step-size proposer --------------------------------------------------
namespace {
int mlp_reserve(sg_ctx* ctx, int n) {
    if (!ctx->mlp_wm) {
        CK(dalloc(&ctx->mlp_wm, SG_MLP_NP));
        CK(dalloc(&ctx->mlp_m1, SG_MLP_NP));
        CK(dalloc(&ctx->mlp_m2, SG_MLP_NP));
        CK(dalloc(&ctx->mlp_grad, SG_MLP_NP));
        CK(dalloc(&ctx->mlp_gpart, (size_t)SG_MLP_NP * 64));
        CK(dalloc(&ctx->mlp_lpart, 64));
        CK(dalloc(&ctx->mlp_loss, 1));
        CK(cudaMalloc(&ctx->mlp_wbf, SG_MLP_NP * 2));
    }
    if (n > ctx->mlp_cap) {
        cudaFree(ctx->mlp_X);
        cudaFree(ctx->mlp_Y);
        cudaFree(ctx->mlp_out);
        cudaFree(ctx->mlp_idx);
        ctx->mlp_X = ctx->mlp_Y = ctx->mlp_out = nullptr;
        ctx->mlp_idx = nullptr;
        CK(dalloc(&ctx->mlp_X, (size_t)n * SG_MLP_IN));
        CK(dalloc(&ctx->mlp_Y, (size_t)n));
        CK(dalloc(&ctx->mlp_out, (size_t)n));
        CK(dalloc(&ctx->mlp_idx, (size_t)n));
        ctx->mlp_cap = n;
    }
    return SG_OK;
}
}  // namespace

extern "C" {

int sg_mlp_param_count(void) { return SG_MLP_NP; }

int sg_mlp_forward(sg_ctx* ctx, int n, const float* X, const float* w, float* out) {
    if (!ctx || n < 0 || (n > 0 && (!X || !w || !out))) return SG_BAD_ARG;
    if (n == 0) return SG_OK;
    CK(cudaSetDevice(ctx->device));
    int st = mlp_reserve(ctx, n);
    if (st != SG_OK) return st;
    CK(cudaMemcpyAsync(ctx->mlp_wm, w, SG_MLP_NP * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    CK(sg_mlp_to_bf16_launch(ctx->mlp_wm, ctx->mlp_wbf, ctx->stream));
    CK(cudaMemcpyAsync(ctx->mlp_X, X, sizeof(float) * n * SG_MLP_IN, cudaMemcpyHostToDevice, ctx->stream));
    CK(sg_mlp_forward_launch(ctx->mlp_wbf, ctx->mlp_X, n, ctx->mlp_out, ctx->stream));
    CK(cudaMemcpyAsync(out, ctx->mlp_out, sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_mlp_grad(sg_ctx* ctx, int n, const float* X, const float* Y, const float* w, float* grad,
                float* loss) {
    if (!ctx || n <= 0 || !X || !Y || !w || !grad || !loss) return SG_BAD_ARG;
    CK(cudaSetDevice(ctx->device));
    int st = mlp_reserve(ctx, n);
    if (st != SG_OK) return st;
    CK(cudaMemcpyAsync(ctx->mlp_wm, w, SG_MLP_NP * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    CK(sg_mlp_to_bf16_launch(ctx->mlp_wm, ctx->mlp_wbf, ctx->stream));
    CK(cudaMemcpyAsync(ctx->mlp_X, X, sizeof(float) * n * SG_MLP_IN, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->mlp_Y, Y, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
    const int nb = std::min(64, std::max(1, n / 32));
    CK(sg_mlp_grad_launch(ctx->mlp_wbf, ctx->mlp_X, ctx->mlp_Y, nullptr, n, ctx->mlp_gpart,
                          ctx->mlp_lpart, nb, ctx->mlp_grad, ctx->mlp_loss, ctx->stream));
    CK(cudaMemcpyAsync(grad, ctx->mlp_grad, SG_MLP_NP * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(loss, ctx->mlp_loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_mlp_train(sg_ctx* ctx, int n, const float* X, const float* Y, int iters, int batch,
                 float lr, uint64_t seed, float* w, float* loss_hist) {
    if (!ctx || n <= 0 || !X || !Y || !w || iters < 0 || batch <= 0) return SG_BAD_ARG;
    CK(cudaSetDevice(ctx->device));
    batch = std::min(batch, n);
    int st = mlp_reserve(ctx, n);
    if (st != SG_OK) return st;
    CK(cudaMemcpyAsync(ctx->mlp_wm, w, SG_MLP_NP * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(ctx->mlp_m1, 0, SG_MLP_NP * sizeof(float), ctx->stream));
    CK(cudaMemsetAsync(ctx->mlp_m2, 0, SG_MLP_NP * sizeof(float), ctx->stream));
    CK(sg_mlp_to_bf16_launch(ctx->mlp_wm, ctx->mlp_wbf, ctx->stream));
    CK(cudaMemcpyAsync(ctx->mlp_X, X, sizeof(float) * n * SG_MLP_IN, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->mlp_Y, Y, sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream));
    // minibatches: a seeded permutation per epoch (splitmix64), uploaded per iteration
    std::vector<int> perm(n), idx(batch);
    for (int i = 0; i < n; i++) perm[i] = i;
    uint64_t s = seed;
    auto next = [&s]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    int pos = n;
    std::vector<float> losses(iters > 0 ? iters : 1);
    const int nb = std::min(64, std::max(1, batch / 32));
    for (int it = 0; it < iters; it++) {
        for (int b = 0; b < batch; b++) {
            if (pos >= n) {
                for (int i = n - 1; i > 0; i--) std::swap(perm[i], perm[next() % (uint64_t)(i + 1)]);
                pos = 0;
            }
            idx[b] = perm[pos++];
        }
        CK(cudaMemcpyAsync(ctx->mlp_idx, idx.data(), sizeof(int) * batch, cudaMemcpyHostToDevice,
                           ctx->stream));
        CK(sg_mlp_grad_launch(ctx->mlp_wbf, ctx->mlp_X, ctx->mlp_Y, ctx->mlp_idx, batch,
                              ctx->mlp_gpart, ctx->mlp_lpart, nb, ctx->mlp_grad, ctx->mlp_loss,
                              ctx->stream));
        CK(sg_mlp_adam_launch(ctx->mlp_wm, ctx->mlp_wbf, ctx->mlp_m1, ctx->mlp_m2, ctx->mlp_grad, lr,
                              it + 1, ctx->stream));
        if (loss_hist)
            CK(cudaMemcpyAsync(&losses[it], ctx->mlp_loss, sizeof(float), cudaMemcpyDeviceToHost,
                               ctx->stream));
        // the index buffer is reused next iteration: wait for this one's upload to land
        CK(cudaStreamSynchronize(ctx->stream));
    }
    CK(cudaMemcpyAsync(w, ctx->mlp_wm, SG_MLP_NP * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (loss_hist)
        for (int it = 0; it < iters; it++) loss_hist[it] = losses[it];
    return SG_OK;
}

int sg_batch_set_proposer(sg_ctx* ctx, const float* w, double safety) {
    if (!ctx || !(safety > 0.0 && safety <= 1.0)) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    drop_graph(ctx);
    if (w) {
        int st = mlp_reserve(ctx, 1);
        if (st != SG_OK) return st;
        CK(cudaMemcpyAsync(ctx->mlp_wm, w, SG_MLP_NP * sizeof(float), cudaMemcpyHostToDevice,
                           ctx->stream));
        CK(sg_mlp_to_bf16_launch(ctx->mlp_wm, P.wbf, ctx->stream));
    }
    const bool was_active = P.log_cap > 0 || P.use_mlp;
    P.use_mlp = w ? 1 : 0;
    P.safety = safety;
    if (!was_active && P.uploaded) {
        int st = proposer_reset(ctx, P);
        if (st != SG_OK) return st;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_batch_set_force_check(sg_ctx* ctx, int every_attempts) {
    if (!ctx || every_attempts < 0) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    P.check_every = every_attempts;
    P.attempt_count = 0;
    return SG_OK;
}

int sg_batch_force_check(sg_ctx* ctx, sg_check_info* out) {
    if (!ctx || !out) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    if (!P.dchk) {
        for (int c = 0; c < P.n_clouds; c++) memset(&out[c], 0, sizeof(sg_check_info));
        return SG_OK;
    }
    std::vector<SgCheck> h(P.n_clouds);
    std::vector<SgCloud> cl(P.n_clouds);
    CK(cudaMemcpyAsync(h.data(), P.dchk, sizeof(SgCheck) * P.n_clouds, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaMemcpyAsync(cl.data(), P.dc, sizeof(SgCloud) * P.n_clouds, cudaMemcpyDeviceToHost,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < P.n_clouds; c++) {
        sg_check_info& o = out[c];
        memset(&o, 0, sizeof o);
        o.max_err = h[c].max_err;
        o.last_err = h[c].last_err;
        o.c_far = h[c].c_far;
        o.kfar = std::sqrt((double)std::min(cl[c].kfar2, h[c].kfar2));
        o.kfar_prior = std::sqrt((double)cl[c].kfar2);
        o.checks = h[c].checks;
        o.probes = h[c].probes;
        o.breaches = h[c].breaches;
        o.max_err_far = h[c].max_kind[0];
        o.max_err_near = h[c].max_kind[1];
        o.max_err_random = h[c].max_kind[2];
        o.worst_err = h[c].worst_err;
        o.worst_rf = h[c].worst_rf;
        o.worst_rn = h[c].worst_rn;
        o.worst_kind = h[c].worst_kind;
        const int wi = h[c].worst_ion;
        o.worst_ion = h[c].worst_err > 0.0 && wi >= 0 && wi < P.n ? P.perm[wi] - cl[c].off : -1;
    }
    return SG_OK;
}

int sg_batch_set_far_threshold(sg_ctx* ctx, double kfar) {
    if (!ctx || !(kfar >= 0.0) || !std::isfinite(kfar)) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    P.kfar_prior = kfar;
    if (P.dchk) {
        std::vector<SgCheck> h0(P.n_clouds);
        for (SgCheck& h : h0) {
            memset(&h, 0, sizeof h);
            h.kfar2 = INFINITY;
        }
        CK(cudaMemcpy(P.dchk, h0.data(), sizeof(SgCheck) * h0.size(), cudaMemcpyHostToDevice));
    }
    return SG_OK;
}

int sg_set_wait_test(sg_ctx* ctx, int tile, int limit_us) {
    if (!ctx || limit_us < 1 || limit_us > 1000000) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    const int w[2] = {tile >= 0 ? tile + 1 : 0, limit_us};
    CK(cudaMemcpyAsync(P.flags + SG_FLAG_WAIT_TILE, w, sizeof w, cudaMemcpyHostToDevice,
                       ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_batch_set_controller_safety(sg_ctx* ctx, double safety) {
    if (!ctx || !(safety > 0.0 && safety <= 1.0)) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    drop_graph(ctx);
    const bool was_active = P.log_cap > 0 || P.use_mlp;
    P.use_mlp = 2;                // proposer kernel: h <- (safety / 0.9) h_controller
    P.safety = safety / 0.9;
    if (!was_active && P.uploaded) {
        int st = proposer_reset(ctx, P);
        if (st != SG_OK) return st;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_batch_set_log(sg_ctx* ctx, int capacity) {
    if (!ctx || capacity < 0) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (P.n_clouds == 0) return SG_NOT_READY;
    CK(cudaSetDevice(ctx->device));
    CK(cudaStreamSynchronize(ctx->stream));
    drop_graph(ctx);
    cudaFree(P.log_feat);
    cudaFree(P.log_num);
    P.log_feat = nullptr;
    P.log_num = nullptr;
    P.log_cap = 0;
    if (capacity > 0) {
        CK(dalloc(&P.log_feat, (size_t)P.n_clouds * capacity * SG_MLP_IN));
        CK(dalloc(&P.log_num, (size_t)P.n_clouds * capacity * 4));
        P.log_cap = capacity;
    }
    if (P.uploaded) {
        int st = proposer_reset(ctx, P);
        if (st != SG_OK) return st;
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return SG_OK;
}

int sg_batch_read_log(sg_ctx* ctx, int cloud, float* feat, double* num, int cap, int* count) {
    if (!ctx || !count) return SG_BAD_ARG;
    Problem& P = ctx->batch;
    if (cloud < 0 || cloud >= P.n_clouds || P.log_cap == 0) return SG_BAD_ARG;
    CK(cudaSetDevice(ctx->device));
    SgProposerState ps;
    CK(cudaMemcpyAsync(&ps, P.pst + cloud, sizeof ps, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const int m = std::min(std::min(ps.logged, P.log_cap), cap);
    if (m > 0 && feat)
        CK(cudaMemcpy(feat, P.log_feat + (size_t)cloud * P.log_cap * SG_MLP_IN,
                      sizeof(float) * m * SG_MLP_IN, cudaMemcpyDeviceToHost));
    if (m > 0 && num)
        CK(cudaMemcpy(num, P.log_num + (size_t)cloud * P.log_cap * 4, sizeof(double) * m * 4,
                      cudaMemcpyDeviceToHost));
    *count = m;
    return SG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// CUNBODY slot (bin/cunbody.h:11-33): one process-wide context on the current device.
// ---------------------------------------------------------------------------
namespace {
std::mutex g_cb_mu;
sg_ctx* g_cb_ctx = nullptr;

int cb_begin(double xj[][3], double mj[], double xi[][3], double eps2, int ni, int nj) {
    if (!g_cb_ctx) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (sg_create(dev, &g_cb_ctx) != SG_OK) return SG_NO_DEVICE;
    }
    sg_ctx* ctx = g_cb_ctx;
    CK(cudaSetDevice(ctx->device));
    if (ni > ctx->cb_ni || nj > ctx->cb_nj) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(ctx->cb_xj);
        cudaFree(ctx->cb_mj);
        cudaFree(ctx->cb_xi);
        cudaFree(ctx->cb_ai);
        if (ctx->cb_host) cudaFreeHost(ctx->cb_host);
        ctx->cb_xj = ctx->cb_mj = ctx->cb_xi = ctx->cb_ai = ctx->cb_host = nullptr;
        ctx->cb_ni = std::max(ni, ctx->cb_ni);
        ctx->cb_nj = std::max(nj, ctx->cb_nj);
        CK(dalloc(&ctx->cb_xj, 3 * (size_t)ctx->cb_nj));
        CK(dalloc(&ctx->cb_mj, (size_t)ctx->cb_nj));
        CK(dalloc(&ctx->cb_xi, 3 * (size_t)ctx->cb_ni));
        CK(dalloc(&ctx->cb_ai, 3 * (size_t)ctx->cb_ni));
        CK(cudaMallocHost((void**)&ctx->cb_host, 3 * sizeof(double) * (size_t)ctx->cb_ni));
    }
    CK(cudaMemcpyAsync(ctx->cb_xj, xj, 3 * sizeof(double) * nj, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->cb_mj, mj, sizeof(double) * nj, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->cb_xi, xi, 3 * sizeof(double) * ni, cudaMemcpyHostToDevice, ctx->stream));
    CK(sg_cunbody_launch(ctx->cb_xj, ctx->cb_mj, ctx->cb_xi, eps2, ctx->cb_ai, ni, nj, ctx->stream));
    CK(cudaMemcpyAsync(ctx->cb_host, ctx->cb_ai, 3 * sizeof(double) * ni, cudaMemcpyDeviceToHost,
                       ctx->stream));
    return SG_OK;
}

int cb_end(double ai[][3], int ni) {
    sg_ctx* ctx = g_cb_ctx;
    if (!ctx) return SG_NOT_READY;
    CK(cudaStreamSynchronize(ctx->stream));
    memcpy(ai, ctx->cb_host, 3 * sizeof(double) * (size_t)ni);
    return SG_OK;
}
}  // namespace

extern "C" {

void cunbody1_force_begin(double xj[][3], double mj[], double xi[][3], double eps2,
                          double ai[][3], int ni, int nj) {
    (void)ai;
    std::lock_guard<std::mutex> lk(g_cb_mu);
    if (ni <= 0) return;
    if (cb_begin(xj, mj, xi, eps2, ni, nj) != SG_OK)
        fprintf(stderr, "simgb: cunbody1_force_begin failed\n");
}

void cunbody1_force_end(double xj[][3], double mj[], double xi[][3], double eps2,
                        double ai[][3], int ni, int nj) {
    (void)xj;
    (void)mj;
    (void)xi;
    (void)eps2;
    (void)nj;
    std::lock_guard<std::mutex> lk(g_cb_mu);
    if (ni <= 0) return;
    if (cb_end(ai, ni) != SG_OK) fprintf(stderr, "simgb: cunbody1_force_end failed\n");
}

void cunbody1_force(double xj[][3], double mj[], double xi[][3], double eps2, double ai[][3],
                    int ni, int nj) {
    cunbody1_force_begin(xj, mj, xi, eps2, ai, ni, nj);
    cunbody1_force_end(xj, mj, xi, eps2, ai, ni, nj);
}

}  // extern "C"
