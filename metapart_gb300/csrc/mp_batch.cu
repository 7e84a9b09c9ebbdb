// Batches: many independent samples partitioned together, each with the results it gets alone.
//
// The reference partitions one input per process launch (metapart.c:3544-4150).  Here the samples of a
// batch share every stage: their FASTQ bytes lie one after another in HBM, their reads take consecutive
// ids (sample q holds [R_q, R_q+1)), their tuples one scan each, one after another (sample-major), and
// one sort orders every sample's tuples at once -- the sample is the most significant part of the key,
// kept by sorting each sample's range on its own (segmented digit passes over the m-mer bucket bits,
// shared-memory unit sorts that never mix samples).  The filter and the union sweep run over all thread
// ranges of all samples, each range with its own sample's initial state; the forests are ranges of one
// parent array (a component never leaves its sample, so its root, the largest id, is the same read as
// alone); the mate union pairs (2j, 2j + 1) never cross samples (every sample has an even read count).
// Each sample's 16 partitions and files follow from its own prefix.  Samples go through the stages in
// groups sized to the HBM budget; the planning between stages (thread ranges, tuple counts) runs on the
// device from the per-sample m-mer histograms, so a group needs a handful of host round trips, not a
// handful per sample.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "k_graph.cuh"
#include "k_kmers.cuh"
#include "k_output.cuh"
#include "k_reads.cuh"
#include "k_sort.cuh"
#include "mp_internal.cuh"

namespace mp {

constexpr uint64_t UMAX32B = 4294967295ull;

// Plan of every sample's single scan (metapart.c:3720-3791 with numScans = 1) and its thread ranges'
// tuple bounds, one thread per sample, from the samples' bucket prefix (shist: nseg * NB + 1 tuple
// offsets).  Restates the host planner (plan_ranges + range_bounds in mp_api.cu) with binary searches:
// threshold i of the walk is the later of the first bucket whose prefix reaches step * i and the bucket
// after the previous threshold.  rb: every sample's T_q + 1 global tuple bounds at rb0[q]; status[q]:
// 0, 1 no k-mers, 2 ranges not covering the scan, 3 ranges not monotone over populated buckets.
constexpr int PLAN_MAX_T = 256;
constexpr int UPLOAD_SEGMENTS = 8;  // upload segments of a group (each parsed and counted as it arrives)

__device__ __forceinline__ uint64_t lower_bound_dev(const uint64_t *h, uint64_t n, uint64_t x)
{
    uint64_t lo = 0, hi = n;
    while (lo < hi) {
        const uint64_t m = (lo + hi) >> 1;
        if (h[m] < x) lo = m + 1; else hi = m;
    }
    return lo;
}

__global__ void k_batch_plan(const uint64_t *shist, int nseg, const uint32_t *T, const uint32_t *rb0, uint64_t *rb,
                             int *status)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nseg) return;
    const uint64_t *h = shist + (uint64_t)q * NB;  // NB + 1 entries: the sample's prefix, offset by its first tuple
    const uint64_t base = h[0], total = h[NB] - base;
    const int Tq = (int)T[q];
    uint64_t *out = rb + rb0[q];
    status[q] = 0;
    if (total == 0) {
        for (int t = 0; t <= Tq; t++) out[t] = base;
        status[q] = 1;
        return;
    }
    // the scan: [0, first bucket whose prefix holds every tuple), NB when the last bucket is populated
    const uint64_t scan_lo = 0, scan_hi = min(lower_bound_dev(h, NB, base + total), (uint64_t)NB);
    // thread ranges: threshold walk with step total / T
    uint32_t thr[PLAN_MAX_T + 1];
    for (int t = 0; t <= Tq; t++) thr[t] = 0;
    const uint64_t step = total / (uint64_t)Tq;
    int64_t prev = -1;
    int cr = 1;
    while (cr <= Tq) {
        const uint64_t lb = lower_bound_dev(h, NB, base + step * (uint64_t)cr);
        const uint64_t i = max(lb, (uint64_t)(prev + 1));
        if (i >= NB) break;
        thr[cr] = cr == Tq ? (uint32_t)scan_hi : (uint32_t)i;
        prev = (int64_t)i;
        cr++;
    }
    if (cr == Tq) thr[cr] = NB;
    // tuple bounds: bin t holds the buckets [M_t, M_t+1), M the running maximum of the range starts
    auto clip = [&](uint64_t x) { return x < scan_lo ? scan_lo : (x > scan_hi ? scan_hi : x); };
    uint64_t M = thr[0];
    const uint64_t m0 = M;
    uint64_t mT = M;
    for (int t = 1; t <= Tq; t++) mT = max(mT, (uint64_t)thr[t]);
    if (h[clip(m0)] != h[scan_lo] || h[scan_hi] != h[clip(mT)]) {
        status[q] = 2;
        return;
    }
    uint64_t acc = base;
    out[0] = base;
    for (int t = 0; t < Tq; t++) {
        const uint64_t Mn = max(M, (uint64_t)thr[t + 1]);
        const uint64_t c = h[clip(Mn)] - h[clip(M)];
        const uint64_t ref = thr[t + 1] > thr[t] ? h[thr[t + 1]] - h[thr[t]] : 0;
        if (ref != c) {
            status[q] = 3;
            return;
        }
        acc += c;
        out[t + 1] = acc;
        M = Mn;
    }
}

}  // namespace mp

using namespace mp;

struct mp_batch {
    mp_ctx *ctx = nullptr;
    int device = 0;
    cudaStream_t st = nullptr, copy_st = nullptr, dl_st = nullptr;  // kernels, uploads, downloads
    DeviceArena arena;  // a group's stage state, released once the group's kernels are queued
    DeviceArena io;     // the groups' FASTQ and partition-file bytes: freed once their copies are done
    double stage_ms[8] = {0};
    int groups = 0;
    double sort_pass_ms = 0;
    uint64_t sort_bytes = 0, sort_tuples = 0;
    int sort_passes = 0;
};

namespace {

struct Sample {
    int idx = 0;                      // position in the caller's arrays
    std::vector<uint64_t> starts;     // chunk starts in the sample's bytes (genFastqIdx)
    std::vector<uint64_t> chunk_rec;  // chunk record starts in the sample's read ids
    uint64_t byte0 = 0;               // where its bytes start in the group's buffer
    uint64_t est = 0;                 // estimated device bytes
};

int sample_error(int code, int q, const char *what)
{
    return set_error(code, "sample %d: %s", q, what);
}

// Device bytes a sample adds to a group: its FASTQ and output, 60 B per read (read table, counts,
// forest, mate-union lists), 36 B per k-mer position (the k-mer cache while enumerating, two tuple
// buffers while sorting), its bucket counts and prefix (12 B per bucket).
uint64_t estimate_sample(const char *fq, uint64_t nbytes, int k)
{
    uint64_t nl[4] = {0, 0, 0, 0};  // the first record's four line ends
    int lines = 0;
    for (uint64_t i = 0; i < nbytes && lines < 4; i++)
        if (fq[i] == '\n') nl[lines++] = i;
    const uint64_t rec = lines == 4 ? nl[3] + 1 : nbytes, L = lines >= 2 ? nl[1] - nl[0] - 1 : 0;
    const uint64_t reads = nbytes / (rec ? rec : 1) + 1;
    const uint64_t pos = L > (uint64_t)k ? reads * (L - (uint64_t)k + 1) : 0;
    return 2 * nbytes + 64 + 60 * reads + 36 * pos + 12ull * NB;
}

}  // namespace

// A group's FASTQ and partition-file buffers whose copies to the host are still queued (done: recorded
// after them on the download stream).
struct PendingIO {
    uint8_t *fq = nullptr, *out = nullptr;
    cudaEvent_t done = nullptr;
};

static void retire(mp_batch *b, PendingIO &x)
{
    if (x.done) {
        cudaEventSynchronize(x.done);
        cudaEventDestroy(x.done);
    }
    b->io.free_persistent(x.fq);
    b->io.free_persistent(x.out);
    x = PendingIO{};
}

// One group of samples through every stage.  Its partition files' copies to the host are queued at the end
// on their own stream and left running (pending); the next group waits for them (as older) once its own
// upload is queued, so the two directions of the host link overlap.
static int run_group(mp_batch *b, const mp_batch_params *p, const mp_batch_sample *smp, std::vector<Sample> &g,
                     PendingIO &older, PendingIO &pending, mp_batch_result *res)
{
    cudaStream_t st = b->st;
    DeviceArena &A = b->arena;
    const int k = p->k, il = p->interleaved ? 1 : 0, nseg = (int)g.size();
    const bool has_hi = 2 * k + 8 > 64;
    int rc = 0;
    struct Release {  // the group's stage state goes back on every return path (stream-ordered frees)
        mp_batch *b;
        ~Release()
        {
            cudaStreamSynchronize(b->copy_st);
            b->arena.release_all();
        }
    } release{b};
    // ---- upload: the samples one after another, each its own copy (the copy stream runs ahead), in
    // segments of consecutive samples of about an eighth of the group's bytes each
    uint64_t total_bytes = 0;
    for (Sample &s : g) {
        s.byte0 = total_bytes;
        total_bytes += smp[s.idx].nbytes;
    }
    std::vector<int> useg{0};  // first sample of every upload segment, then nseg
    {
        uint64_t acc = 0;
        for (int q = 0; q < nseg; q++) {
            acc += smp[g[q].idx].nbytes;
            if (q + 1 < nseg && acc * UPLOAD_SEGMENTS >= total_bytes * useg.size()) useg.push_back(q + 1);
        }
        useg.push_back(nseg);
    }
    const int nu = (int)useg.size() - 1;
    uint8_t *d_fq = b->io.alloc_persistent<uint8_t>(total_bytes + 64);
    pending.fq = d_fq;  // from here on the caller frees it
    if (!d_fq) return set_error(MP_ENOMEM, "device memory for a group's %llu FASTQ bytes", (unsigned long long)total_bytes);
    Events ev(nu + 1, cudaEventDisableTiming);
    cudaEventRecord(ev[nu], st);
    MP_CUDA(cudaStreamWaitEvent(b->copy_st, ev[nu], 0));
    for (int u = 0; u < nu; u++) {
        for (int q = useg[u]; q < useg[u + 1]; q++) {
            const mp_batch_sample &s = smp[g[q].idx];
            MP_CUDA(cudaMemcpyAsync(d_fq + g[q].byte0, s.fastq, s.nbytes, cudaMemcpyHostToDevice, b->copy_st));
        }
        cudaEventRecord(ev[u], b->copy_st);
    }
    MP_CUDA(cudaMemsetAsync(d_fq + total_bytes, 0, 64, st));
    // the previous group's files go down while this group's bytes go up (the link carries both ways at
    // once); the parse waits for them, since its small read-backs would queue behind the big copies
    retire(b, older);
    // ---- per upload segment, as its bytes arrive: parse, the samples' and their chunks' first records,
    // k-mer cache and per-sample bucket counts
    uint32_t *cc = A.alloc_persistent<uint32_t>((size_t)nseg * NB);
    uint32_t *err = A.alloc_persistent<uint32_t>(1);
    uint64_t *d_srec = A.alloc_persistent<uint64_t>(nseg + nu);  // each segment's sample read offsets (local)
    if (!cc || !err || !d_srec) return set_error(MP_ENOMEM, "device memory for a group's bucket counts");
    MP_CUDA(cudaMemsetAsync(cc, 0, (size_t)nseg * NB * sizeof(uint32_t), st));
    MP_CUDA(cudaMemsetAsync(err, 0, 4, st));
    std::vector<ParsedReads> prs(nu);
    std::vector<KcPiece> kc(nu);
    std::vector<uint64_t> R(nseg + 1, 0), RU(nu + 1, 0);
    for (int u = 0; u < nu; u++) {
        const int qa = useg[u], qb = useg[u + 1];
        const uint64_t b0 = g[qa].byte0, b1 = g[qb - 1].byte0 + smp[g[qb - 1].idx].nbytes;
        MP_CUDA(cudaStreamWaitEvent(st, ev[u], 0));
        {
            StageTimer tm(st, b->stage_ms, 0);
            rc = parse_fastq_range(d_fq, b0, b1, &prs[u], A, st);
        }
        if (rc) {  // name the sample: parse the segment's samples one by one until one fails
            const std::string msg = mp_last_error();
            for (int q = qa; q < qb; q++) {
                ParsedReads one;
                const int r1 = parse_fastq_range(d_fq, g[q].byte0, g[q].byte0 + smp[g[q].idx].nbytes, &one, A, st);
                A.free_persistent(one.rec_start);
                A.free_persistent(one.seq_off);
                A.free_persistent(one.seq_len);
                if (r1) return sample_error(r1, g[q].idx, mp_last_error());
            }
            return set_error(rc, "samples %d..%d: %s", g[qa].idx, g[qb - 1].idx, msg.c_str());
        }
        // every sample's chunk starts (its first is its own start, its last its end), relative to the segment
        std::vector<uint64_t> qs, qr;
        for (int q = qa; q < qb; q++)
            for (uint64_t x : g[q].starts) qs.push_back(g[q].byte0 - b0 + x);
        qr.assign(qs.size(), 0);
        rc = records_at_offsets(&prs[u], qs.data(), (int)qs.size(), qr.data(), A, st);
        for (int q = qa, at = 0; q < qb; q++) {
            const int nq = (int)g[q].starts.size();
            for (int c = 0; c < nq; c++)
                if (qr[at + c] == ~0ull)
                    return sample_error(MP_EFMT, g[q].idx, c == nq - 1 ? "the FASTQ does not end on a record end"
                                                                     : "a chunk does not start on a record");
            g[q].chunk_rec.assign(nq, 0);
            for (int c = 0; c < nq; c++) g[q].chunk_rec[c] = qr[at + c] - qr[at];
            const uint64_t n = g[q].chunk_rec[nq - 1];
            if (il && (n & 1)) return sample_error(MP_EFMT, g[q].idx, "interleaved input with an odd record count");
            if (n & 1) return sample_error(MP_EUNSUP, g[q].idx, "the mate union needs an even read count");
            if (il)
                for (int c = 0; c + 1 < nq; c++)
                    if ((g[q].chunk_rec[c + 1] - g[q].chunk_rec[c]) & 1)
                        return sample_error(MP_EFMT, g[q].idx, "an interleaved chunk has an odd record count");
            R[q + 1] = R[q] + n;
            at += nq;
        }
        if (rc) return rc;
        RU[u + 1] = R[qb];
        StageTimer tm(st, b->stage_ms, 1);
        if (!make_kc_piece(A, st, prs[u], RU[u], k, &kc[u]))
            return set_error(MP_ENOMEM, "device memory for the k-mer cache of samples %d..%d", g[qa].idx, g[qb - 1].idx);
        std::vector<uint64_t> loc(qb - qa + 1);
        for (int q = qa; q <= qb; q++) loc[q - qa] = R[q] - RU[u];
        uint64_t *dl = d_srec + qa + u;
        MP_CUDA(cudaMemcpyAsync(dl, loc.data(), loc.size() * 8, cudaMemcpyHostToDevice, st));
        launch_count(d_fq + b0, prs[u], k, 0, dl, qb - qa, cc + (size_t)qa * NB, nullptr, err, st, kc[u].off, kc[u].lo,
                     kc[u].hi);
    }
    const uint64_t N = R[nseg];
    if (N >= UMAX32B) return set_error(MP_EUNSUP, "a group of more than 2^32 - 2 reads");
    // ---- one read table for the group, global read ids
    ParsedReads pr;
    {
        StageTimer tm(st, b->stage_ms, 0);
        pr.n_reads = N;
        pr.rec_start = A.alloc_persistent<uint64_t>(N + 1);
        pr.seq_off = A.alloc_persistent<uint64_t>(N + 1);
        pr.seq_len = A.alloc_persistent<uint32_t>(N + 1);
        if (!pr.rec_start || !pr.seq_off || !pr.seq_len) return set_error(MP_ENOMEM, "device memory for the read table");
        for (int u = 0; u < nu; u++) concat_records(prs[u], g[useg[u]].byte0, pr, RU[u], st);
    }
    for (auto &x : prs) {
        A.free_persistent(x.rec_start);
        A.free_persistent(x.seq_off);
        A.free_persistent(x.seq_len);
    }
    // ---- every sample's bucket prefix and scan plan on the device
    uint64_t *shist = A.alloc_persistent<uint64_t>((size_t)nseg * NB + 1);
    std::vector<uint32_t> hT(nseg), hrb0(nseg + 1, 0);
    for (int q = 0; q < nseg; q++) {
        hT[q] = (uint32_t)smp[g[q].idx].num_threads;
        hrb0[q + 1] = hrb0[q] + hT[q];
    }
    const int Rn = (int)hrb0[nseg];
    uint32_t *dT = A.alloc<uint32_t>(nseg), *drb0 = A.alloc<uint32_t>(nseg + 1);
    uint64_t *drb = A.alloc<uint64_t>(Rn + 1);
    int *dstat = A.alloc<int>(nseg);
    const size_t tbh = scan_tmp_bytes((size_t)nseg * NB);
    void *tmph = A.alloc<uint8_t>(tbh);
    if (!shist || !dT || !drb0 || !drb || !dstat || !tmph) return set_error(MP_ENOMEM, "device memory for the group's plan");
    std::vector<uint64_t> rb(Rn + 1);
    std::vector<int> hstat(nseg);
    uint32_t herr = 0;
    {
        StageTimer tm(st, b->stage_ms, 1);
        scan_u32_to_u64(cc, shist, (size_t)nseg * NB, shist + (size_t)nseg * NB, tmph, tbh, st);
        MP_CUDA(cudaMemcpyAsync(dT, hT.data(), nseg * 4, cudaMemcpyHostToDevice, st));
        MP_CUDA(cudaMemcpyAsync(drb0, hrb0.data(), (nseg + 1) * 4, cudaMemcpyHostToDevice, st));
        (count_launch(), k_batch_plan<<<(nseg + 63) / 64, 64, 0, st>>>(shist, nseg, dT, drb0, drb, dstat));
        MP_CUDA(cudaMemcpyAsync(rb.data(), drb, (Rn + 1) * 8, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaMemcpyAsync(hstat.data(), dstat, nseg * sizeof(int), cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaStreamSynchronize(st));
        MP_CUDA(cudaGetLastError());
    }
    A.free_persistent(cc);
    A.release_scratch();
    if (herr & DERR_LONG_READ) return set_error(MP_EUNSUP, "a read is longer than %d bases", MAX_READ_COUNT);
    for (int q = 0; q < nseg; q++) {
        if (hstat[q] == 1) return sample_error(MP_EUNSUP, g[q].idx, "the histogram holds no k-mers");
        if (hstat[q] == 2) return sample_error(MP_EUNSUP, g[q].idx, "thread k-mer ranges do not cover the scan's populated buckets");
        if (hstat[q] == 3) return sample_error(MP_EUNSUP, g[q].idx, "thread k-mer ranges are not monotone over populated buckets");
    }
    SortSegments segs;
    segs.nseg = nseg;
    segs.tstart.resize(nseg + 1);
    for (int q = 0; q < nseg; q++) segs.tstart[q] = rb[hrb0[q]];
    segs.tstart[nseg] = rb[Rn];
    const uint64_t T_all = rb[Rn];
    // ---- enumeration: every k-mer of every read (one scan per sample), read order
    SortBufs sb;
    {
        StageTimer tm(st, b->stage_ms, 2);
        uint32_t *cnt = A.alloc<uint32_t>(N + 1), *d_b = A.alloc<uint32_t>(2);
        uint64_t *off = A.alloc<uint64_t>(N + 2), *ntot = A.alloc<uint64_t>(1);
        const size_t tb = scan_tmp_bytes(N + 1);
        void *tmp = A.alloc<uint8_t>(tb);
        if (!cnt || !d_b || !off || !ntot || !tmp) return set_error(MP_ENOMEM, "device memory for enumeration offsets");
        const uint32_t hb[2] = {0, NB};
        MP_CUDA(cudaMemcpyAsync(d_b, hb, 8, cudaMemcpyHostToDevice, st));
        for (const KcPiece &q : kc)
            if (q.n && launch_kc_count_scans(q.off, q.lo, q.hi, q.n, k, d_b, 1, cnt + q.r0, N + 1, err, st))
                return set_error(MP_EARG, "enumeration count");
        MP_CUDA(cudaMemsetAsync(cnt + N, 0, 4, st));
        scan_u32_to_u64(cnt, off, N + 1, ntot, tmp, tb, st);
        uint64_t n = 0;
        MP_CUDA(cudaMemcpyAsync(&n, ntot, 8, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaStreamSynchronize(st));
        if (herr & DERR_LONG_READ) return set_error(MP_EUNSUP, "a read has 300 or more k-mer positions");
        if (herr & DERR_TOO_MANY)
            return set_error(MP_EUNSUP, "a read has 256 or more k-mers (the reference counts them in 8 bits, "
                                        "enumerateKmers.c:152)");
        if (n != T_all)
            return set_error(MP_EFMT, "the group enumerates %llu tuples but its histograms hold %llu", (unsigned long long)n,
                             (unsigned long long)T_all);
        for (int x = 0; x < 2; x++) {
            sb.lo[x] = A.alloc_persistent<uint64_t>(n + 1);
            sb.id[x] = A.alloc_persistent<uint32_t>(n + 1);
            sb.hi[x] = has_hi ? A.alloc_persistent<uint8_t>(n + 1) : nullptr;
            if (!sb.lo[x] || !sb.id[x] || (has_hi && !sb.hi[x]))
                return set_error(MP_ENOMEM, "device memory for %llu tuples", (unsigned long long)n);
        }
        for (const KcPiece &q : kc)
            launch_kc_write(q.off, q.lo, q.hi, q.r0, q.n, k, 0, NB, nullptr, off, sb.lo[0], sb.hi[0], sb.id[0], st);
        for (auto &x : kc) free_kc_piece(A, x);
        A.release_scratch();
    }
    // ---- sort: every sample's tuples by (k-mer, adjacency), within the sample's range
    int lo_buf = 0, hi_buf = 0;
    {
        StageTimer tm(st, b->stage_ms, 3);
        SortStats ss;
        if ((rc = bucket_sort(sb, T_all, has_hi, k, shist, 0, (uint64_t)nseg * NB, A, st, &ss, &lo_buf, &hi_buf, &segs)))
            return rc;
        b->sort_pass_ms += ss.pass_ms;
        b->sort_bytes += ss.bytes;
        b->sort_passes += ss.passes;
        b->sort_tuples += T_all;
        A.release_scratch();
    }
    Tuples tp;
    tp.lo = sb.lo[lo_buf];
    tp.hi = has_hi ? sb.hi[hi_buf] : nullptr;
    tp.id = sb.id[lo_buf];
    tp.n = T_all;
    // free the other buffer's big arrays (the filter and the union read only the sorted ones)
    A.free_persistent(sb.lo[lo_buf ^ 1]);
    A.free_persistent(sb.id[lo_buf ^ 1]);
    if (has_hi) A.free_persistent(sb.hi[hi_buf ^ 1]);
    // ---- filter and unions over every thread range of every sample
    uint32_t *parent = A.alloc_persistent<uint32_t>(N + 1), *size = A.alloc_persistent<uint32_t>(N + 1);
    uint8_t *filtered = A.alloc_persistent<uint8_t>(N + 1);
    if (!parent || !size || !filtered) return set_error(MP_ENOMEM, "device memory for the forest");
    launch_init_parent(parent, N, st);
    MP_CUDA(cudaMemsetAsync(filtered, 0, N + 1, st));
    {
        StageTimer tm(st, b->stage_ms, 4);
        if ((rc = filter_scan(tp, rb, parent, filtered, A, st, false, true))) return rc;
    }
    {
        std::vector<uint32_t> rseg(Rn);
        for (int q = 0; q < nseg; q++)
            for (uint32_t t = hrb0[q]; t < hrb0[q + 1]; t++) rseg[t] = (uint32_t)q;
        StageTimer tm(st, b->stage_ms, 5);
        if ((rc = union_segments(tp, rb, rseg, segs.tstart, parent, filtered, N, A, st))) return rc;
    }
    A.release_scratch();
    A.free_persistent(sb.lo[lo_buf]);
    A.free_persistent(sb.id[lo_buf]);
    if (has_hi) A.free_persistent(sb.hi[hi_buf]);
    A.free_persistent(shist);
    // ---- mate union and every sample's partitions
    std::vector<uint64_t> bounds((size_t)nseg * 17);
    {
        StageTimer tm(st, b->stage_ms, 6);
        int rounds = 0;
        if ((rc = mate_union(parent, N, size, A, st, &rounds))) return rc;
        if ((rc = plan_partitions_segments(parent, size, N, R, bounds.data(), A, st))) return rc;
        A.release_scratch();
    }
    // ---- partition files: planned for all samples at once, built in HBM in batches of entries, each
    // batch's bytes going down to the samples' buffers on the copy stream while the next is built
    OutputPlan plan;
    std::vector<uint64_t> fsz, file0;
    std::vector<std::vector<uint64_t>> crec(nseg);
    std::vector<int> Ts(nseg);
    for (int q = 0; q < nseg; q++) {
        crec[q] = g[q].chunk_rec;
        Ts[q] = smp[g[q].idx].num_threads;
    }
    {
        StageTimer tm(st, b->stage_ms, 7);
        if ((rc = plan_output_batch(pr, parent, il, R, bounds, crec, Ts, &plan, fsz, file0, A, st))) return rc;
        A.release_scratch();
    }
    std::vector<uint64_t> fb(fsz.size() + 1, 0);  // byte offset of every global file
    for (size_t f = 0; f < fsz.size(); f++) fb[f + 1] = fb[f] + fsz[f];
    for (int q = 0; q < nseg; q++) {
        const mp_batch_sample &s = smp[g[q].idx];
        const uint64_t tot = fb[file0[q + 1]] - fb[file0[q]];
        if (s.out && s.out_cap < tot) return sample_error(MP_EARG, g[q].idx, "output buffer too small");
        mp_batch_result &r = res[g[q].idx];
        r.status = 0;
        r.error[0] = 0;
        r.n_reads = R[q + 1] - R[q];
        r.out_total = tot;
        memcpy(r.bounds, &bounds[(size_t)q * 17], sizeof r.bounds);
        if (s.file_sizes) memcpy(s.file_sizes, &fsz[file0[q]], 16ull * Ts[q] * sizeof(uint64_t));
    }
    // labels first (the forest goes back with the group's stage state)
    for (int q = 0; q < nseg; q++) {
        const mp_batch_sample &s = smp[g[q].idx];
        const uint64_t n = R[q + 1] - R[q];
        if (!s.labels) continue;
        if (s.labels_cap < n) return sample_error(MP_EARG, g[q].idx, "labels buffer too small");
        MP_CUDA(cudaMemcpyAsync(s.labels, parent + R[q], n * 4, cudaMemcpyDeviceToHost, st));
    }
    MP_CUDA(cudaStreamSynchronize(st));
    for (int q = 0; q < nseg; q++) {  // labels in each sample's own read ids
        const mp_batch_sample &s = smp[g[q].idx];
        if (!s.labels) continue;
        const uint64_t n = R[q + 1] - R[q];
        for (uint64_t x = 0; x < n; x++) s.labels[x] -= (uint32_t)R[q];
    }
    uint8_t *d_out = b->io.alloc_persistent<uint8_t>(plan.total + 16);
    if (!d_out) return set_error(MP_ENOMEM, "device memory for the output bytes");
    pending.out = d_out;
    {
        constexpr int KB = 8;
        StageTimer tm(st, b->stage_ms, 7);
        uint64_t e[KB + 1], o[KB + 1];
        for (int x = 0; x <= KB; x++) e[x] = plan.n * (uint64_t)x / KB;
        for (int x = 0; x < KB; x++)
            if (e[x] < plan.n) MP_CUDA(cudaMemcpyAsync(&o[x], plan.off + e[x], 8, cudaMemcpyDeviceToHost, st));
        MP_CUDA(cudaStreamSynchronize(st));
        for (int x = 0; x < KB; x++)
            if (e[x] >= plan.n) o[x] = plan.total;
        o[KB] = plan.total;
        Events bev(KB, cudaEventDisableTiming);
        for (int x = 0; x < KB; x++) {
            if ((rc = copy_output_range(plan, e[x], e[x + 1], d_fq, d_out, st))) return rc;
            cudaEventRecord(bev[x], st);
            MP_CUDA(cudaStreamWaitEvent(b->dl_st, bev[x], 0));
            for (int q = 0; q < nseg; q++) {  // the part of each sample's bytes this batch built
                const mp_batch_sample &s = smp[g[q].idx];
                const uint64_t s0 = fb[file0[q]], s1 = fb[file0[q + 1]];
                const uint64_t a = std::max(s0, o[x]), z = std::min(s1, o[x + 1]);
                if (s.out && a < z)
                    MP_CUDA(cudaMemcpyAsync(s.out + (a - s0), d_out + a, z - a, cudaMemcpyDeviceToHost, b->dl_st));
            }
        }
        // the copies to the host run on during the next group's kernels; the buffers wait for them
        MP_CUDA(cudaEventCreateWithFlags(&pending.done, cudaEventDisableTiming));
        MP_CUDA(cudaEventRecord(pending.done, b->dl_st));
        MP_CUDA(cudaGetLastError());
    }
    b->groups++;
    return 0;
}

extern "C" {

int mp_batch_create(mp_ctx *ctx, mp_batch **out)
{
    if (!ctx || !out) return set_error(MP_EARG, "null argument");
    const int dev = ctx_device(ctx);
    MP_CUDA(cudaSetDevice(dev));
    mp_batch *b = new mp_batch;
    b->ctx = ctx;
    b->device = dev;
    if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->copy_st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->dl_st, cudaStreamNonBlocking) != cudaSuccess) {
        if (b->st) cudaStreamDestroy(b->st);
        if (b->copy_st) cudaStreamDestroy(b->copy_st);
        delete b;
        return set_error(MP_ECUDA, "cannot create a stream");
    }
    b->arena.st = b->st;
    b->io.st = b->st;
    ctx_budget(ctx, &b->arena.budget_used, &b->arena.budget_limit);
    ctx_budget(ctx, &b->io.budget_used, &b->io.budget_limit);
    *out = b;
    return 0;
}

void mp_batch_destroy(mp_batch *b)
{
    if (!b) return;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->copy_st);
    cudaStreamSynchronize(b->dl_st);
    b->arena.release_all();
    b->io.release_all();
    cudaStreamSynchronize(b->st);
    cudaStreamDestroy(b->st);
    cudaStreamDestroy(b->copy_st);
    cudaStreamDestroy(b->dl_st);
    delete b;
}

int mp_batch_run(mp_batch *b, const mp_batch_params *p, int nsamples, const mp_batch_sample *samples,
                 mp_batch_result *results)
{
    if (!b || !p || !samples || !results || nsamples < 1) return set_error(MP_EARG, "bad argument");
    if (p->k < 11 || p->k > 31) return set_error(MP_EARG, "k must be in [11, 31]");
    MP_CUDA(cudaSetDevice(b->device));
    for (int q = 0; q < nsamples; q++) {
        results[q] = mp_batch_result{};
        results[q].status = MP_EARG;
        snprintf(results[q].error, sizeof results[q].error, "not run");
    }
    for (auto &v : b->stage_ms) v = 0;
    b->groups = 0;
    b->sort_pass_ms = 0;
    b->sort_bytes = b->sort_tuples = 0;
    b->sort_passes = 0;
    // chunk index of every sample (genFastqIdx) and its footprint estimate
    std::vector<Sample> all(nsamples);
    for (int q = 0; q < nsamples; q++) {
        const mp_batch_sample &s = samples[q];
        if (!s.fastq || s.nbytes == 0 || s.num_chunks < 1 || s.num_threads < 1 || s.num_threads > PLAN_MAX_T)
            return sample_error(MP_EARG, q, "bad sample (bytes, chunks, or numThreads outside [1, 256])");
        std::vector<int32_t> fno(s.num_chunks + 1);
        std::vector<uint64_t> ofs(s.num_chunks + 1);
        int cnt = 0;
        const char *files[1] = {s.fastq};
        const uint64_t sizes[1] = {s.nbytes};
        int rc = mp_fastq_index(s.num_chunks, 0, p->interleaved ? 0 : 1, p->interleaved ? 1 : 0, 1, files, sizes, fno.data(),
                                ofs.data(), &cnt);
        if (rc) return sample_error(rc, q, mp_last_error());
        if (cnt < 2 || ofs[0] != 0) return sample_error(MP_EFMT, q, "too short for a chunk index");
        if ((cnt - 1) % s.num_threads) return sample_error(MP_EARG, q, "numThreads must divide the number of chunks");
        all[q].idx = q;
        all[q].starts.assign(ofs.begin(), ofs.begin() + cnt);
        all[q].est = estimate_sample(s.fastq, s.nbytes, p->k);
    }
    // groups: consecutive samples while their estimated bytes fit what the budget or the device has left
    uint64_t avail = 0;
    {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) == cudaSuccess) avail = fr;
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, b->device) == cudaSuccess) {
            uint64_t rsv = 0, used = 0;
            if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &rsv) == cudaSuccess &&
                cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && rsv > used)
                avail += rsv - used;
        }
        cudaGetLastError();
        if (b->arena.budget_used && b->arena.budget_limit != ~0ull) {
            const uint64_t u = b->arena.budget_used->load();
            avail = std::min<uint64_t>(avail, u < b->arena.budget_limit ? b->arena.budget_limit - u : 0);
        }
        const char *e = getenv("MP_BATCH_GROUP_BYTES");  // a smaller group size (tests)
        if (e && *e) avail = std::min<uint64_t>(avail, strtoull(e, nullptr, 10));
        avail = avail / 10 * 9;
    }
    std::vector<std::vector<Sample>> groups;
    uint64_t acc = 0;
    for (int q = 0; q < nsamples; q++) {
        const uint64_t need = all[q].est + (256ull << 20);
        if (groups.empty() || acc + need > avail) {
            groups.emplace_back();
            acc = 0;
        }
        groups.back().push_back(all[q]);
        acc += need;
    }
    // groups one after another on the device; group g - 1's files go down while group g's bytes go up
    PendingIO prev, cur;
    int rc = 0;
    for (size_t gi = 0; gi < groups.size() && !rc; gi++) {
        rc = run_group(b, p, samples, groups[gi], prev, cur, results);
        retire(b, prev);  // (already done inside, unless the group failed early)
        prev = cur;
        cur = PendingIO{};
        if (rc)
            for (const Sample &s : groups[gi]) {
                results[s.idx].status = rc;
                snprintf(results[s.idx].error, sizeof results[s.idx].error, "%s", mp_last_error());
            }
    }
    // every copy to the host is done before the call returns; a failure leaves nothing behind
    const std::string msg = rc ? std::string(mp_last_error()) : std::string();
    retire(b, prev);
    cudaStreamSynchronize(b->copy_st);
    cudaStreamSynchronize(b->dl_st);
    b->io.release_all();
    const cudaError_t e = cudaStreamSynchronize(b->st);
    if (!rc && e != cudaSuccess) rc = set_cuda_error(e, "mp_batch_run", __FILE__, __LINE__);
    if (rc && !msg.empty()) set_error(rc, "%s", msg.c_str());
    return rc;
}

int mp_batch_stage_ms(const mp_batch *b, double *ms, int n)
{
    if (!b || !ms) return set_error(MP_EARG, "null argument");
    for (int i = 0; i < n && i < 8; i++) ms[i] = b->stage_ms[i];
    return 0;
}

int mp_batch_groups(const mp_batch *b) { return b ? b->groups : 0; }

int mp_batch_set_wait_limits(mp_batch *b, uint32_t lookback_spins, uint32_t union_retries, uint32_t mate_rounds)
{
    if (!b) return set_error(MP_EARG, "null batch");
    const WaitLimits d;
    b->arena.lim.lookback_spins = lookback_spins ? lookback_spins : d.lookback_spins;
    b->arena.lim.union_retries = union_retries ? union_retries : d.union_retries;
    b->arena.lim.mate_rounds = mate_rounds ? mate_rounds : d.mate_rounds;
    return 0;
}

int mp_batch_sort_stats(const mp_batch *b, uint64_t *tuples, int *passes, double *pass_ms, uint64_t *bytes)
{
    if (!b) return set_error(MP_EARG, "null batch");
    if (tuples) *tuples = b->sort_tuples;
    if (passes) *passes = b->sort_passes;
    if (pass_ms) *pass_ms = b->sort_pass_ms;
    if (bytes) *bytes = b->sort_bytes;
    return 0;
}

}  // extern "C"
