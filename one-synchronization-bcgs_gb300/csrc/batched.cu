// Batched BCGSI+P-1S: many independent tall-skinny QRs (each the reference's
// bcgsi2P1s, SRC/orth.c:48-222, on its own X and R) in one captured CUDA graph.
//
// The plan lays every matrix's per-block-step operations on a common sequence of
// stages:
//   TSQR of block 1 (one launch per tree level, one for the root sign fixes, one
//   per down-sweep level), then the first step (Gram W, Cholesky, update U_2,
//   Gram G, small ops, update Q_2), then per block step i: update U_i, the step's
//   one Gram (partials + fixed-order reduction), the small s x s operations, and
//   update Q_i.
// Each stage is ONE launch over all matrices that have it (persistent over the
// stage's CTAs: a CTA finds its matrix through the stage's prefix array), and the
// whole sequence is captured once into a CUDA graph that orth_gb300_batch_run
// replays. The small operations of a step (Cholesky of the corrected Gram, the R
// block, the reconstruction of the next step's coefficients and its Cholesky) run
// in one CTA per matrix; none of them reads what the following update writes, so
// they run before it. Every matrix sees exactly the operations, operands and
// summation orders of the single-matrix driver: with the same Gram chunking
// (orth_gb300_set_gram_chunk_rows) the results are bit-identical.
//
// Tuning: per block size s, the Gram's B-panel width (8, 16 or 32 columns; the
// A-panel holds 512 / width columns, 64 threads per CTA) and the rows per Gram
// chunk (4096 ... 32768) are picked by timing each candidate on a representative
// Gram stage of that class's matrices.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/orth_gb300.h"
#include "batched.h"
#include "common.cuh"
#include "kernels.h"
#include "split.h"

namespace bcgs {

int tsqr_tile_batched_prepare();
int split_batch_enqueue(int variant, int count, const int* m, const int* n, const int* s, double* const* dX,
                        const long long* ldX, double* const* dR, const int* ldR, int precision, cudaStream_t st,
                        int* dstatus, int max_slots);
bool split_supported(i64 m, int n, int s);

namespace {

constexpr int kTR = 256;                // TSQR tile rows for nc <= 32
constexpr int kMaxS = 16;
constexpr int kClasses = 3;             // s <= 4, s <= 8, s <= 16
constexpr int kRowsMin = 4096;          // smallest Gram chunk candidate
constexpr int kTbCand[3] = {8, 16, 32};
constexpr int kRowsCand[4] = {4096, 8192, 16384, 32768};

int class_of(int s) { return s <= 4 ? 0 : (s <= 8 ? 1 : 2); }

struct Mat {
    i64 m, ld;
    int n, s, p;
    double* X;
    double* R;
    int ldR;
    int cls;
    // workspace
    double *G1, *G2, *Scol, *Sd, *Yd, *part, *tsqr;
    int* status;
};

enum StageKind { kStGram = 0, kStSmall, kStUpd, kStTile, kStRoot, kStApply };

struct Stage {
    int kind;
    size_t job_off, prefix_off, prefix2_off;   // byte offsets into the job blob
    int njobs, items, items2;                  // items2: the Gram reduction's CTAs
};

// A Gram request of one matrix in one stage (filled into a GramJob once the
// matrix class's panel and chunk rows are known).
struct GramReq {
    int mat;
    int na, b0, nb;
    double* C;
    int ldc;
};

struct Blob {
    std::vector<char> bytes;
    template <class T>
    size_t put(const std::vector<T>& v) {
        size_t off = (bytes.size() + 15) & ~(size_t)15;
        bytes.resize(off + v.size() * sizeof(T));
        if (!v.empty()) std::memcpy(bytes.data() + off, v.data(), v.size() * sizeof(T));
        return off;
    }
};

i64 small_block_doubles(int n, int s) { return 2LL * (n + s) * 2 * s + (i64)n * s + 3LL * s * s + 64; }

i64 tsqr_doubles(i64 m, int s) { return tsqr_workspace_doubles(m, s); }

i64 part_doubles_of(i64 m, int n, int s) {
    return ceil_div(m, kRowsMin) * (i64)(n + s) * (2 * s) + 64;
}

}  // namespace

struct BatchPlan {
    int count = 0;
    std::vector<Mat> mats;
    int tb[kClasses] = {16, 16, 32};
    int rows[kClasses] = {8192, 8192, 8192};
    bool tuned = false;
    // device memory: workspace (per-matrix blocks + status) and the job blob
    void* ws = nullptr;
    size_t ws_bytes = 0;
    void* jobs_dev = nullptr;
    size_t jobs_bytes = 0;
    std::vector<Stage> stages;
    std::vector<std::vector<GramReq>> gram_reqs;   // per Gram stage, in stage order
    std::vector<int> gram_stage_idx;
    cudaStream_t own_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;
    int graph_nodes = 0;
    // Split-precision batches: staged graphs per wave (BCGSI+P-1S, s <= 16), or the
    // single-matrix driver per matrix on concurrent streams.
    bool split = false;
    SplitStaged* staged = nullptr;
    int variant = 0, precision = 0, max_slots = 0;
    std::vector<int> vm, vn, vs, vldR;
    std::vector<double*> vX, vR;
    std::vector<long long> vldX;
    int* dstatus = nullptr;   // 8 ints per matrix: status words, split error word
};

namespace {

// Per-matrix workspace layout; returns total bytes (doubles, then the status ints).
size_t layout_workspace(BatchPlan& P, char* base) {
    size_t off = 0;
    auto take = [&](size_t bytes) -> char* {
        off = (off + 255) & ~(size_t)255;
        char* p = base ? base + off : nullptr;
        off += bytes;
        return p;
    };
    for (Mat& M : P.mats) {
        double* sb = (double*)take((size_t)small_block_doubles(M.n, M.s) * sizeof(double));
        const int n = M.n, s = M.s;
        M.G1 = sb;
        M.G2 = sb ? M.G1 + (i64)(n + s) * 2 * s : nullptr;
        M.Scol = sb ? M.G2 + (i64)(n + s) * 2 * s : nullptr;
        double* S0 = sb ? M.Scol + (i64)n * s : nullptr;
        M.Sd = sb ? S0 + (i64)s * s : nullptr;
        M.Yd = sb ? M.Sd + (i64)s * s : nullptr;
        M.part = (double*)take((size_t)part_doubles_of(M.m, M.n, M.s) * sizeof(double));
        M.tsqr = (double*)take((size_t)tsqr_doubles(M.m, M.s) * sizeof(double));
    }
    int* st = (int*)take((size_t)P.count * kStatusWords * sizeof(int));
    for (int b = 0; b < P.count; ++b) P.mats[b].status = st ? st + (size_t)b * kStatusWords : nullptr;
    return off + 256;
}

// Shape of the Gram of block step i (0: the first step's second Gram), by the
// schedule's rule (SRC/orth.c:125-133, 177-199).
void step_gram_shape(const Mat& M, int i, int& na, int& b0, int& nb) {
    const int s = M.s, n = M.n;
    if (i == 0) {
        const int nZ = std::min(s, n - 2 * s);
        na = 2 * s + nZ; b0 = s; nb = s + nZ;
        return;
    }
    const int mScol = (i + 1) * s;
    if (i < M.p - 1) {
        const int nZn = std::min(s, n - (i + 2) * s);
        na = mScol + s + nZn; b0 = mScol; nb = s + nZn;
    } else {
        const int nZ = std::min(s, n - (i + 1) * s);
        na = mScol + nZ; b0 = mScol; nb = nZ;
    }
}

GramJob make_gram_job(const Mat& M, const GramReq& q, int tb, int rows) {
    GramJob J;
    J.X = M.X; J.ld = M.ld; J.m = M.m;
    J.na = q.na; J.b0 = q.b0; J.nb = q.nb;
    i64 nch = ceil_div(M.m, rows);
    if (nch < 1) nch = 1;
    J.nchunks = (int)nch;
    i64 rpc = ceil_div(M.m, nch);
    J.rows_per_chunk = ceil_div(rpc, 32) * 32;   // the single-matrix driver's rule
    J.part = M.part;
    J.C = q.C; J.ldc = q.ldc;
    J.tb = tb;
    J.tilesA = (int)ceil_div(q.na, gram_batched_panel_rows(tb));
    J.tilesB = (int)ceil_div(q.nb, tb);
    return J;
}

// Builds every stage of the schedule (jobs + prefix arrays in `blob`).
void build_schedule(BatchPlan& P, Blob& blob) {
    P.stages.clear();
    P.gram_reqs.clear();
    P.gram_stage_idx.clear();
    const int B = P.count;
    std::vector<Mat>& mats = P.mats;

    auto add_prefixed = [&](int kind, auto& jobs, const std::vector<int>& counts, int items2) {
        Stage S;
        S.kind = kind;
        S.njobs = (int)jobs.size();
        std::vector<int> prefix(jobs.size() + 1, 0);
        for (size_t j = 0; j < jobs.size(); ++j) prefix[j + 1] = prefix[j] + counts[j];
        S.items = prefix.back();
        S.items2 = items2;
        S.job_off = blob.put(jobs);
        S.prefix_off = blob.put(prefix);
        S.prefix2_off = 0;
        if (S.njobs > 0) P.stages.push_back(S);
    };
    auto add_gram = [&](std::vector<GramReq>& reqs) {
        if (reqs.empty()) return;
        std::vector<GramJob> jobs;
        std::vector<int> counts;
        for (const GramReq& q : reqs) {
            const Mat& M = mats[q.mat];
            GramJob J = make_gram_job(M, q, P.tb[M.cls], P.rows[M.cls]);
            jobs.push_back(J);
            counts.push_back(J.nchunks * J.tilesA * J.tilesB);
        }
        P.gram_stage_idx.push_back((int)P.stages.size());
        P.gram_reqs.push_back(reqs);
        Stage S;
        S.kind = kStGram;
        S.njobs = (int)jobs.size();
        std::vector<int> prefix(jobs.size() + 1, 0), prefix2(jobs.size() + 1, 0);
        for (size_t j = 0; j < jobs.size(); ++j) {
            prefix[j + 1] = prefix[j] + counts[j];
            prefix2[j + 1] = prefix2[j] + (int)ceil_div((i64)reqs[j].na * reqs[j].nb, 256);
        }
        S.items = prefix.back();
        S.items2 = prefix2.back();
        S.job_off = blob.put(jobs);
        S.prefix_off = blob.put(prefix);
        S.prefix2_off = blob.put(prefix2);
        P.stages.push_back(S);
    };
    auto add_small = [&](std::vector<SmallJob>& jobs) {
        if (jobs.empty()) return;
        std::vector<int> counts(jobs.size(), 1);
        add_prefixed(kStSmall, jobs, counts, 0);
    };
    auto add_upd = [&](std::vector<UpdJob>& jobs) {
        if (jobs.empty()) return;
        std::vector<int> counts;
        for (const UpdJob& J : jobs) counts.push_back((int)ceil_div(J.m, 128));
        add_prefixed(kStUpd, jobs, counts, 0);
    };
    auto pyth = [](const double* Om, int ldom, const double* A, int lda, int k, int nz, double* T, int step) {
        SmallSub S{};
        S.kind = kSmallPyth;
        S.p0 = Om; S.ld0 = ldom; S.p1 = A; S.ld1 = lda; S.a = k; S.b = nz; S.out = T; S.ldo = nz; S.step = step;
        return S;
    };
    auto scol = [](const double* G, int ldg, int mZ, int s, int nZ, const double* Yd, double* Scol) {
        SmallSub S{};
        S.kind = kSmallScol;
        S.p0 = G; S.ld0 = ldg; S.a = mZ; S.b = s; S.c = nZ; S.p1 = Yd; S.ld1 = s; S.out = Scol; S.ldo = mZ + s;
        return S;
    };
    auto rblock = [](int c0, int K, int ny, const double* A, int lda, const double* Bm, int ldb, const double* Sd,
                     const double* Yd) {
        SmallSub S{};
        S.kind = kSmallRblock;
        S.a = c0; S.b = K; S.c = ny; S.d = 0;
        S.p0 = A; S.ld0 = lda; S.p1 = Bm; S.ld1 = ldb; S.p2 = Sd; S.ld2 = ny; S.p3 = Yd; S.ld3 = ny;
        return S;
    };
    auto upd = [](const Mat& M, int K, int c0, int nc, const double* S, int lds, const double* T, int ldt) {
        UpdJob J;
        J.X = M.X; J.ld = M.ld; J.m = M.m; J.q0 = 0; J.K = K; J.c0 = c0; J.nc = nc;
        J.S = S; J.lds = lds; J.T = T; J.ldt = ldt;
        return J;
    };

    // ---- TSQR of block 1 (the single-panel tree of launch_tsqr, per matrix) ----
    struct Lv { double* ptr; i64 rows, ld; };
    std::vector<std::vector<Lv>> lv(B);
    std::vector<double*> rroot(B);
    int Lmax = 0;
    for (int b = 0; b < B; ++b) {
        Mat& M = mats[b];
        lv[b].push_back({M.X, M.m, M.ld});
        double* cursor = M.tsqr;
        while (lv[b].back().rows > kTR) {
            const i64 tiles = ceil_div(lv[b].back().rows, kTR);
            double* next = cursor;
            cursor = cursor ? cursor + tiles * M.s * M.s : nullptr;
            lv[b].push_back({next, tiles * M.s, tiles * M.s});
        }
        rroot[b] = cursor;
        Lmax = std::max(Lmax, (int)lv[b].size() - 1);
    }
    for (int l = 0; l <= Lmax; ++l) {
        std::vector<TsqrTileJob> jobs;
        std::vector<int> counts;
        for (int b = 0; b < B; ++b) {
            const int L = (int)lv[b].size() - 1;
            if (l > L) continue;
            const Lv& v = lv[b][l];
            TsqrTileJob J;
            J.A = v.ptr; J.lda = v.ld; J.rows = v.rows; J.nc = mats[b].s;
            if (l < L) {
                const i64 tiles = ceil_div(v.rows, kTR);
                J.Rst = lv[b][l + 1].ptr; J.ldr = tiles * mats[b].s;
                counts.push_back((int)tiles);
            } else {
                J.Rst = rroot[b]; J.ldr = mats[b].s;
                counts.push_back(1);
            }
            jobs.push_back(J);
        }
        add_prefixed(kStTile, jobs, counts, 0);
    }
    {
        std::vector<TsqrRootJob> jobs;
        std::vector<int> counts;
        for (int b = 0; b < B; ++b) {
            const Lv& v = lv[b].back();
            TsqrRootJob J;
            J.Q = v.ptr; J.ldq = v.ld; J.hq = (int)v.rows; J.nc = mats[b].s;
            J.R = rroot[b]; J.ldr = mats[b].s; J.Rout = mats[b].R; J.ldro = mats[b].ldR;
            jobs.push_back(J);
            counts.push_back(1);
        }
        add_prefixed(kStRoot, jobs, counts, 0);
    }
    for (int l = Lmax - 1; l >= 0; --l) {
        std::vector<TsqrApplyJob> jobs;
        std::vector<int> counts;
        for (int b = 0; b < B; ++b) {
            const int L = (int)lv[b].size() - 1;
            if (l >= L) continue;
            TsqrApplyJob J;
            J.Q = lv[b][l].ptr; J.ldq = lv[b][l].ld; J.rows = lv[b][l].rows; J.nc = mats[b].s; J.TR = kTR;
            J.P = lv[b][l + 1].ptr; J.ldp = lv[b][l + 1].ld;
            jobs.push_back(J);
            counts.push_back((int)ceil_div(J.rows, 128));
        }
        add_prefixed(kStApply, jobs, counts, 0);
    }

    // ---- First block step (SRC/orth.c:110-147) ----
    std::vector<int> nZ(B), na1(B);
    {
        std::vector<GramReq> g;
        for (int b = 0; b < B; ++b) {
            const Mat& M = mats[b];
            g.push_back({b, 2 * M.s, M.s, M.s, M.G2, 2 * M.s});                       // :111-114
        }
        add_gram(g);
        std::vector<SmallJob> sj;
        for (int b = 0; b < B; ++b) {
            const Mat& M = mats[b];
            SmallJob J{};
            J.status = M.status; J.R = M.R; J.ldR = M.ldR;
            J.sub[0] = pyth(M.G2 + M.s, 2 * M.s, M.G2, 2 * M.s, M.s, M.s, M.Sd, 1);     // :115-119
            J.nsub = 1;
            sj.push_back(J);
        }
        add_small(sj);
        std::vector<UpdJob> uj;
        for (int b = 0; b < B; ++b) {
            const Mat& M = mats[b];
            uj.push_back(upd(M, M.s, M.s, M.s, M.G2, 2 * M.s, M.Sd, M.s));               // :121-124
        }
        add_upd(uj);
        g.clear();
        for (int b = 0; b < B; ++b) {
            const Mat& M = mats[b];
            const int s = M.s;
            nZ[b] = M.n - 2 * s < s ? M.n - 2 * s : s;                                   // :125
            na1[b] = 2 * s + nZ[b];
            g.push_back({b, na1[b], s, s + nZ[b], M.G1, na1[b]});                        // :127-133
        }
        add_gram(g);
        sj.clear();
        for (int b = 0; b < B; ++b) {
            const Mat& M = mats[b];
            const int s = M.s, na = na1[b];
            SmallJob J{};
            J.status = M.status; J.R = M.R; J.ldR = M.ldR;
            J.sub[0] = pyth(M.G1 + s, na, M.G1, na, s, s, M.Yd, 1);                       // :134-137
            J.sub[1] = rblock(s, s, s, M.G2, 2 * s, M.G1, na, M.Sd, M.Yd);               // :144-147
            J.nsub = 2;
            if (M.p > 1) {
                const int mScol = 2 * s;
                J.sub[2] = scol(M.G1, na, s, s, nZ[b], M.Yd, M.Scol);                    // :155-159
                J.sub[3] = pyth(M.G1 + mScol + (i64)s * na, na, M.Scol, mScol, mScol, nZ[b], M.Sd, 2);   // :160-171
                J.nsub = 4;
            }
            sj.push_back(J);
        }
        add_small(sj);
        uj.clear();
        for (int b = 0; b < B; ++b) {
            const Mat& M = mats[b];
            uj.push_back(upd(M, M.s, M.s, M.s, M.G1, na1[b], M.Yd, M.s));                // :139-142
        }
        add_upd(uj);
    }

    // ---- Block steps i = 1 .. p-1 (SRC/orth.c:152-218) ----
    int Pmax = 0;
    for (const Mat& M : mats) Pmax = std::max(Pmax, M.p);
    std::vector<int> mZ(B);
    for (int b = 0; b < B; ++b) mZ[b] = mats[b].s;
    for (int i = 1; i < Pmax; ++i) {
        std::vector<UpdJob> uU, uQ;
        std::vector<GramReq> g;
        std::vector<SmallJob> sj;
        std::vector<int> nY(B, 0), nZn(B, 0), na(B, 0);
        for (int b = 0; b < B; ++b) {
            const Mat& M = mats[b];
            if (i >= M.p) continue;
            const int s = M.s, n = M.n, mScol = mZ[b] + s;
            uU.push_back(upd(M, mScol, mScol, nZ[b], M.Scol, mScol, M.Sd, nZ[b]));     // :173-176
            int nb;
            if (i < M.p - 1) {                                                           // :177-190
                nZn[b] = n - (i + 1) * s - s < s ? n - (i + 1) * s - s : s;
                na[b] = mScol + s + nZn[b];
                nb = s + nZn[b];
                nY[b] = s;
            } else {                                                                     // :191-199
                nZn[b] = nZ[b];
                na[b] = mScol + nZ[b];
                nb = nZ[b];
                nY[b] = nZ[b];
            }
            g.push_back({b, na[b], mScol, nb, M.G1, na[b]});                             // the one sync
        }
        add_upd(uU);
        add_gram(g);
        for (int b = 0; b < B; ++b) {
            const Mat& M = mats[b];
            if (i >= M.p) continue;
            const int s = M.s, mScol = mZ[b] + s, lg = na[b];
            SmallJob J{};
            J.status = M.status; J.R = M.R; J.ldR = M.ldR;
            J.sub[0] = pyth(M.G1 + mScol, lg, M.G1, lg, mScol, nY[b], M.Yd, i + 1);    // :200-204
            J.sub[1] = rblock(mScol, mScol, nY[b], M.Scol, mScol, M.G1, lg, M.Sd, M.Yd);  // :211-215
            J.nsub = 2;
            if (i + 1 < M.p) {
                // Start of step i+1 (:155-171): they read G, Yd and write Scol, Sd,
                // none of which the update of Q_i below touches.
                const int mZ2 = mScol, mScol2 = mZ2 + s;
                J.sub[2] = scol(M.G1, lg, mZ2, s, nZn[b], M.Yd, M.Scol);
                J.sub[3] = pyth(M.G1 + mScol2 + (i64)s * lg, lg, M.Scol, mScol2, mScol2, nZn[b], M.Sd, i + 2);
                J.nsub = 4;
            }
            sj.push_back(J);
            uQ.push_back(upd(M, mScol, mScol, nY[b], M.G1, lg, M.Yd, nY[b]));           // :206-209
        }
        add_small(sj);
        add_upd(uQ);
        for (int b = 0; b < B; ++b) {
            if (i >= mats[b].p) continue;
            mZ[b] += mats[b].s;
            nZ[b] = nZn[b];
        }
    }
}

int enqueue_all(BatchPlan& P, cudaStream_t st) {
    const char* base = (const char*)P.jobs_dev;
    long long l0 = g_launch_count;
    cudaError_t ce = (cudaError_t)zero_async(P.mats[0].status, (size_t)P.count * kStatusWords * sizeof(int), st);
    if (ce != cudaSuccess) return (int)ce;
    for (const Stage& S : P.stages) {
        const int* prefix = (const int*)(base + S.prefix_off);
        int rc = 0;
        switch (S.kind) {
            case kStGram: {
                const GramJob* jobs = (const GramJob*)(base + S.job_off);
                rc = launch_gram_partial_batched(jobs, prefix, S.njobs, S.items, st);
                if (!rc)
                    rc = launch_gram_reduce_batched(jobs, (const int*)(base + S.prefix2_off), S.njobs, S.items2, st);
                break;
            }
            case kStSmall:
                rc = launch_small_batched((const SmallJob*)(base + S.job_off), S.njobs, st);
                break;
            case kStUpd:
                rc = launch_update_batched((const UpdJob*)(base + S.job_off), prefix, S.njobs, S.items, st);
                break;
            case kStTile:
                rc = launch_tsqr_tile_batched((const TsqrTileJob*)(base + S.job_off), prefix, S.njobs, S.items,
                                              kMaxS, st);
                break;
            case kStRoot:
                rc = launch_tsqr_root_batched((const TsqrRootJob*)(base + S.job_off), S.njobs, st);
                break;
            case kStApply:
                rc = launch_tsqr_apply_batched((const TsqrApplyJob*)(base + S.job_off), prefix, S.njobs, S.items,
                                               kMaxS, st);
                break;
        }
        if (rc) return rc;
    }
    P.launches = g_launch_count - l0;
    return 0;
}

int upload_schedule(BatchPlan& P) {
    Blob blob;
    build_schedule(P, blob);
    if (P.jobs_dev) cudaFree(P.jobs_dev);
    P.jobs_dev = nullptr;
    P.jobs_bytes = blob.bytes.size();
    BCGS_CUDA_TRY(cudaMalloc(&P.jobs_dev, P.jobs_bytes + 16));
    BCGS_CUDA_TRY(cudaMemcpy(P.jobs_dev, blob.bytes.data(), P.jobs_bytes, cudaMemcpyHostToDevice));
    return 0;
}

// Times the Gram of each class's matrices at their middle block step for every
// (panel width, chunk rows) candidate and keeps the fastest.
int autotune(BatchPlan& P, cudaStream_t st) {
    cudaEvent_t e0, e1;
    BCGS_CUDA_TRY(cudaEventCreate(&e0));
    BCGS_CUDA_TRY(cudaEventCreate(&e1));
    int rc = 0;
    for (int c = 0; c < kClasses && !rc; ++c) {
        std::vector<GramReq> reqs;
        for (int b = 0; b < P.count && reqs.size() < 256; ++b) {
            const Mat& M = P.mats[b];
            if (M.cls != c) continue;
            int na, b0, nb;
            step_gram_shape(M, M.p > 1 ? std::max(1, (M.p - 1) / 2) : 0, na, b0, nb);
            reqs.push_back({b, na, b0, nb, M.G1, na});
        }
        if (reqs.empty()) continue;
        float best = 1e30f;
        for (int tb : kTbCand) {
            for (int rows : kRowsCand) {
                std::vector<GramJob> jobs;
                std::vector<int> prefix(1, 0), prefix2(1, 0);
                for (const GramReq& q : reqs) {
                    GramJob J = make_gram_job(P.mats[q.mat], q, tb, rows);
                    jobs.push_back(J);
                    prefix.push_back(prefix.back() + J.nchunks * J.tilesA * J.tilesB);
                    prefix2.push_back(prefix2.back() + (int)ceil_div((i64)q.na * q.nb, 256));
                }
                Blob blob;
                const size_t jo = blob.put(jobs), po = blob.put(prefix), p2 = blob.put(prefix2);
                void* d = nullptr;
                if ((rc = (int)cudaMalloc(&d, blob.bytes.size()))) break;
                rc = (int)cudaMemcpy(d, blob.bytes.data(), blob.bytes.size(), cudaMemcpyHostToDevice);
                float ms = 0.f;
                for (int rep = 0; rep < 2 && !rc; ++rep) {
                    cudaEventRecord(e0, st);
                    rc = launch_gram_partial_batched((const GramJob*)((char*)d + jo), (const int*)((char*)d + po),
                                                     (int)jobs.size(), prefix.back(), st);
                    if (!rc)
                        rc = launch_gram_reduce_batched((const GramJob*)((char*)d + jo), (const int*)((char*)d + p2),
                                                        (int)jobs.size(), prefix2.back(), st);
                    cudaEventRecord(e1, st);
                    if (!rc) rc = (int)cudaEventSynchronize(e1);
                    if (!rc) rc = (int)cudaEventElapsedTime(&ms, e0, e1);
                }
                cudaFree(d);
                if (rc) break;
                if (ms < best) { best = ms; P.tb[c] = tb; P.rows[c] = rows; }
            }
            if (rc) break;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    P.tuned = (rc == 0);
    return rc;
}

void free_plan(BatchPlan* P) {
    if (!P) return;
    if (P->staged) split_staged_destroy(P->staged);
    if (P->dstatus) cudaFree(P->dstatus);
    if (P->exec) cudaGraphExecDestroy(P->exec);
    if (P->graph) cudaGraphDestroy(P->graph);
    if (P->jobs_dev) cudaFree(P->jobs_dev);
    if (P->ws) cudaFree(P->ws);
    if (P->own_stream) cudaStreamDestroy(P->own_stream);
    delete P;
}

int fill_mats(BatchPlan& P, int count, const int* m, const int* n, const int* s, double* const* dX,
              const long long* ldX, double* const* dR, const int* ldR) {
    P.count = count;
    P.mats.resize(count);
    for (int b = 0; b < count; ++b) {
        Mat& M = P.mats[b];
        M.m = m[b]; M.n = n[b]; M.s = s[b];
        M.X = dX ? dX[b] : nullptr; M.ld = ldX ? ldX[b] : m[b];
        M.R = dR ? dR[b] : nullptr; M.ldR = ldR ? ldR[b] : n[b];
        if (M.s < 1 || M.s > kMaxS || M.n < 2 * M.s || M.m < M.n || M.ld < M.m || M.ldR < M.n) return 2;
        M.p = (M.n - M.s + M.s - 1) / M.s;
        M.cls = class_of(M.s);
    }
    return 0;
}

}  // namespace
}  // namespace bcgs

using bcgs::BatchPlan;

struct orth_gb300_batch {
    BatchPlan* plan;
};

extern "C" {

int orth_gb300_batch_create(orth_gb300_batch** out, int variant, int count, const int* m, const int* n,
                            const int* s, double* const* dX, const long long* ldX, double* const* dR,
                            const int* ldR, int precision, int flags, void* stream) {
    using namespace bcgs;
    if (!out) return 2;
    *out = nullptr;
    if (count < 1 || !m || !n || !s || !dX || !dR) return 2;
    for (int b = 0; b < count; ++b)
        if (!dX[b] || !dR[b]) return 2;
    if (precision == ORTH_GB300_SPLIT_BF16 || precision == ORTH_GB300_SPLIT_BF16_FAST) {
        if (variant < ORTH_GB300_BCGSI2P1S || variant > ORTH_GB300_BCGSI2P2S) return 4;
        BatchPlan* P = new BatchPlan();
        P->split = true; P->variant = variant; P->precision = precision; P->count = count;
        P->max_slots = (flags & ORTH_GB300_BATCH_ONE_STREAM) ? 1 : 0;
        for (int b = 0; b < count; ++b) {
            const long long lx = ldX ? ldX[b] : m[b];
            const int lr = ldR ? ldR[b] : n[b];
            if (s[b] < 1 || n[b] < 2 * s[b] || m[b] < n[b] || lx < m[b] || lr < n[b]) { free_plan(P); return 2; }
            if (!split_supported(m[b], n[b], s[b])) { free_plan(P); return 4; }
            P->vm.push_back(m[b]); P->vn.push_back(n[b]); P->vs.push_back(s[b]);
            P->vX.push_back(dX[b]); P->vR.push_back(dR[b]); P->vldX.push_back(lx); P->vldR.push_back(lr);
        }
        if (cudaMalloc(&P->dstatus, (size_t)count * 8 * sizeof(int)) != cudaSuccess ||
            cudaMemset(P->dstatus, 0, (size_t)count * 8 * sizeof(int)) != cudaSuccess) {
            free_plan(P);
            return 3;
        }
        if (!(flags & (ORTH_GB300_BATCH_ONE_STREAM | ORTH_GB300_BATCH_STREAMS)) &&
            split_staged_supported(variant, count, s)) {
            const int rc = split_staged_create(count, m, n, s, dX, ldX, dR, ldR,
                                               precision == ORTH_GB300_SPLIT_BF16_FAST ? 6 : 7, P->dstatus, -1,
                                               (cudaStream_t)stream, &P->staged);
            if (rc) { free_plan(P); return rc; }
            long long k = 0;
            int nodes = 0;
            split_staged_info(P->staged, &k, nullptr, &nodes, nullptr);
            P->launches = k;
            P->graph_nodes = nodes;
        }
        *out = new orth_gb300_batch{P};
        return 0;
    }
    if (variant != ORTH_GB300_BCGSI2P1S || precision != ORTH_GB300_FP64) return 4;
    BatchPlan* P = new BatchPlan();
    int rc = fill_mats(*P, count, m, n, s, dX, ldX, dR, ldR);
    if (rc) { free_plan(P); return rc; }
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = tsqr_tile_batched_prepare()) != 0) { free_plan(P); return 3; }
    P->ws_bytes = layout_workspace(*P, nullptr);
    if (cudaMalloc(&P->ws, P->ws_bytes) != cudaSuccess) { free_plan(P); return 3; }
    layout_workspace(*P, (char*)P->ws);
    if (cudaStreamCreateWithFlags(&P->own_stream, cudaStreamNonBlocking) != cudaSuccess) { free_plan(P); return 3; }
    if (!st) st = P->own_stream;
    if (flags & ORTH_GB300_BATCH_TUNE) {
        if (autotune(*P, st)) { free_plan(P); return 3; }
    }
    if (upload_schedule(*P)) { free_plan(P); return 3; }
    // Capture the whole batched QR once; runs replay it.
    cudaStream_t cs = P->own_stream;
    if (cudaStreamSynchronize(st) != cudaSuccess) { free_plan(P); return 3; }
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { free_plan(P); return 3; }
    rc = enqueue_all(*P, cs);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(cs, &g);
    if (rc || ce != cudaSuccess || !g) { if (g) cudaGraphDestroy(g); free_plan(P); return 3; }
    P->graph = g;
    if (cudaGraphInstantiate(&P->exec, g, 0) != cudaSuccess) { free_plan(P); return 3; }
    size_t nodes = 0;
    cudaGraphGetNodes(g, nullptr, &nodes);
    P->graph_nodes = (int)nodes;
    orth_gb300_batch* h = new orth_gb300_batch{P};
    *out = h;
    return 0;
}

int orth_gb300_batch_run(orth_gb300_batch* h, void* stream) {
    if (!h || !h->plan) return 2;
    cudaStream_t st = (cudaStream_t)stream;
    if (h->plan->staged) return bcgs::split_staged_run(h->plan->staged, st);
    if (h->plan->split) {
        BatchPlan& P = *h->plan;
        const long long l0 = bcgs::g_launch_count;
        const int rc = bcgs::split_batch_enqueue(P.variant, P.count, P.vm.data(), P.vn.data(), P.vs.data(),
                                                 P.vX.data(), P.vldX.data(), P.vR.data(), P.vldR.data(),
                                                 P.precision, st, P.dstatus, P.max_slots);
        P.launches = bcgs::g_launch_count - l0;
        return rc;
    }
    if (!h->plan->exec) return 2;
    if (cudaGraphLaunch(h->plan->exec, st) != cudaSuccess) return 3;
    bcgs::g_launch_count += h->plan->launches;
    return 0;
}

int orth_gb300_batch_status(orth_gb300_batch* h, int* breakdown_step, int* breakdown_info, int* nbroken) {
    using namespace bcgs;
    if (!h || !h->plan) return 2;
    BatchPlan& P = *h->plan;
    if (cudaDeviceSynchronize() != cudaSuccess) return 3;
    const int stride = P.split ? 8 : kStatusWords;
    std::vector<int> st((size_t)P.count * stride);
    const int* src = P.split ? P.dstatus : P.mats[0].status;
    if (cudaMemcpy(st.data(), src, st.size() * sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
    int broken = 0, timeouts = 0;
    for (int b = 0; b < P.count; ++b) {
        if (breakdown_step) breakdown_step[b] = st[(size_t)b * stride];
        if (breakdown_info) breakdown_info[b] = st[(size_t)b * stride + 1];
        if (st[(size_t)b * stride]) ++broken;
        if (P.split && st[(size_t)b * stride + 4]) ++timeouts;
    }
    if (timeouts) return 3;   // a bounded wait of the split kernels ran out
    if (nbroken) *nbroken = broken;
    return 0;
}

int orth_gb300_batch_info(const orth_gb300_batch* h, long long* launches_per_run, long long* workspace_bytes,
                          int* graph_nodes, int* tuned) {
    using namespace bcgs;
    if (!h || !h->plan) return 2;
    const BatchPlan& P = *h->plan;
    if (launches_per_run) *launches_per_run = P.launches;
    if (workspace_bytes) *workspace_bytes = (long long)(P.ws_bytes + P.jobs_bytes);
    if (P.staged && workspace_bytes) split_staged_info(P.staged, nullptr, workspace_bytes, nullptr, nullptr);
    if (graph_nodes) *graph_nodes = P.graph_nodes;
    if (tuned)
        for (int c = 0; c < kClasses; ++c) { tuned[2 * c] = P.tb[c]; tuned[2 * c + 1] = P.rows[c]; }
    return 0;
}

void orth_gb300_batch_destroy(orth_gb300_batch* h) {
    if (!h) return;
    bcgs::free_plan(h->plan);
    delete h;
}

int orth_gb300_split_batch_dry_run(int count, const int* m, const int* n, const int* s, long long budget_bytes,
                                   int* waves, long long* launches_per_run, long long* wave_bytes) {
    if (count < 1 || !m || !n || !s) return 2;
    if (!bcgs::split_staged_supported(ORTH_GB300_BCGSI2P1S, count, s)) return 4;
    return bcgs::split_staged_dry_run(count, m, n, s, budget_bytes, waves, launches_per_run, wave_bytes);
}

int orth_gb300_batch_dry_run(int count, const int* m, const int* n, const int* s, long long* stages,
                             long long* launches_per_run, long long* workspace_bytes) {
    using namespace bcgs;
    if (count < 1 || !m || !n || !s) return 2;
    BatchPlan P;
    int rc = fill_mats(P, count, m, n, s, nullptr, nullptr, nullptr, nullptr);
    if (rc) return rc;
    const size_t wsb = layout_workspace(P, nullptr);
    Blob blob;
    build_schedule(P, blob);
    long long launches = 0;
    for (const Stage& S : P.stages) launches += (S.kind == kStGram) ? 2 : 1;
    if (stages) *stages = (long long)P.stages.size();
    if (launches_per_run) *launches_per_run = launches;
    if (workspace_bytes) *workspace_bytes = (long long)(wsb + blob.bytes.size());
    return 0;
}

}  // extern "C"
