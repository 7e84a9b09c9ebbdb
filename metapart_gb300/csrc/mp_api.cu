// C ABI of libmetapart_gpu.so (include/metapart_gpu.h): contexts, jobs and the stage drivers.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "k_graph.cuh"
#include "k_kmers.cuh"
#include "k_output.cuh"
#include "k_reads.cuh"
#include "k_sort.cuh"
#include "mp_internal.cuh"

namespace mp {

static thread_local std::string g_err;

int set_error(int code, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

int set_cuda_error(cudaError_t e, const char *what, const char *file, int line)
{
    return set_error(MP_ECUDA, "%s: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
}

constexpr uint64_t UMAX32 = 4294967295ull;

static std::atomic<uint64_t> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int sm_count()
{
    static std::atomic<int> cached[64];
    int dev = 0;
    cudaGetDevice(&dev);
    std::atomic<int> &c = cached[dev & 63];
    int n = c.load(std::memory_order_relaxed);
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        n = 1;
    }
    c.store(n, std::memory_order_relaxed);
    return n;
}

__global__ void k_init_parent(uint32_t *parent, uint64_t n)
{
    const uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x < n) parent[x] = (uint32_t)x;
}

void launch_init_parent(uint32_t *parent, uint64_t n, cudaStream_t st)
{
    if (n) (count_launch(), k_init_parent<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(parent, n));
}

void free_kc_piece(DeviceArena &arena, KcPiece &q)
{
    arena.free_persistent(q.off);
    arena.free_persistent(q.lo);
    arena.free_persistent(q.hi);
    arena.free_persistent(q.poff);
    arena.free_persistent(q.pw);
    arena.free_persistent(q.pn);
    q = KcPiece{};
}

bool make_pk_piece(DeviceArena &arena, cudaStream_t st, const ParsedReads &pr, uint64_t r0, int k, KcPiece *out)
{
    const uint64_t N = pr.n_reads;
    KcPiece q;
    q.r0 = r0;
    q.n = N;
    uint32_t *nr = arena.alloc<uint32_t>(N + 1);
    uint64_t *tot = arena.alloc<uint64_t>(1);
    size_t tb = scan_tmp_bytes(N + 1);
    void *tmp = arena.alloc<uint8_t>(tb);
    q.poff = arena.alloc_persistent<uint64_t>(N + 2);
    uint64_t P = 0;
    bool ok = nr && tot && tmp && q.poff;
    if (ok) {
        launch_pk_rounds(pr, k, nr, st);
        ok = cudaMemsetAsync(nr + N, 0, 4, st) == cudaSuccess;
    }
    if (ok) {
        scan_u32_to_u64(nr, q.poff, N + 1, tot, tmp, tb, st);
        ok = cudaMemcpyAsync(&P, tot, 8, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaStreamSynchronize(st) == cudaSuccess;
    }
    if (ok) {
        q.pw = arena.alloc_persistent<uint64_t>(P + 1);
        q.pn = arena.alloc_persistent<uint32_t>(P + 1);
        ok = q.pw && q.pn;
    }
    arena.free_scratch(nr);
    arena.free_scratch(tot);
    arena.free_scratch(tmp);
    if (!ok) {
        free_kc_piece(arena, q);
        return false;
    }
    *out = q;
    return true;
}

// The enumeration over one piece of the count pass's copy of the reads (either form): every scan's
// per-read tuple counts (cnt indexed by global read id), and one bucket range's tuples at off.
int store_count_scans(const KcPiece &q, const uint32_t *seq_len, int k, const uint32_t *bounds, int S, uint32_t *cnt,
                      uint64_t stride, uint32_t *err, cudaStream_t st)
{
    if (!q.n) return 0;
    if (q.pw) return launch_pk_count_scans(q.poff, q.pw, q.pn, q.r0, q.n, seq_len, k, bounds, S, cnt, stride, err, st);
    return launch_kc_count_scans(q.off, q.lo, q.hi, q.n, k, bounds, S, cnt + q.r0, stride, err, st);
}

void store_write(const KcPiece &q, const uint32_t *seq_len, int k, uint32_t lo, uint32_t hi, const uint32_t *label,
                 const uint64_t *off, uint64_t *o_lo, uint8_t *o_hi, uint32_t *o_id, uint32_t *err, cudaStream_t st)
{
    if (q.pw) launch_pk_write(q.poff, q.pw, q.pn, q.r0, q.n, seq_len, k, lo, hi, label, off, o_lo, o_hi, o_id, err, st);
    else launch_kc_write(q.off, q.lo, q.hi, q.r0, q.n, k, lo, hi, label, off, o_lo, o_hi, o_id, st);
}

bool make_kc_piece(DeviceArena &arena, cudaStream_t st, const ParsedReads &pr, uint64_t r0, int k, KcPiece *out)
{
    const uint64_t N = pr.n_reads;
    KcPiece q;
    q.r0 = r0;
    q.n = N;
    uint32_t *npos = arena.alloc<uint32_t>(N + 1);
    uint64_t *tot = arena.alloc<uint64_t>(1);
    size_t tb = scan_tmp_bytes(N + 1);
    void *tmp = arena.alloc<uint8_t>(tb);
    q.off = arena.alloc_persistent<uint64_t>(N + 2);
    uint64_t P = 0;
    bool ok = npos && tot && tmp && q.off;
    if (ok) {
        launch_kc_positions(pr, k, npos, st);
        ok = cudaMemsetAsync(npos + N, 0, 4, st) == cudaSuccess;
    }
    if (ok) {
        scan_u32_to_u64(npos, q.off, N + 1, tot, tmp, tb, st);
        ok = cudaMemcpyAsync(&P, tot, 8, cudaMemcpyDeviceToHost, st) == cudaSuccess &&
             cudaStreamSynchronize(st) == cudaSuccess;
    }
    if (ok) {
        q.lo = arena.alloc_persistent<uint64_t>(P + 1);
        q.hi = arena.alloc_persistent<uint8_t>(P + 1);
        ok = q.lo && q.hi;
    }
    arena.free_scratch(npos);
    arena.free_scratch(tot);
    arena.free_scratch(tmp);
    if (!ok) {
        free_kc_piece(arena, q);
        return false;
    }
    *out = q;
    return true;
}

}  // namespace mp

using namespace mp;

struct mp_ctx {
    int device = 0;
    uint64_t budget = ~0ull;
    std::atomic<uint64_t> used{0};
    std::mutex mu;
};

int mp::ctx_device(const mp_ctx *ctx) { return ctx->device; }

void mp::ctx_budget(mp_ctx *ctx, std::atomic<uint64_t> **used, uint64_t *limit)
{
    *used = &ctx->used;
    *limit = ctx->budget;
}

struct mp_job {
    mp_ctx *ctx = nullptr;
    cudaStream_t st = nullptr;
    DeviceArena arena;
    uint8_t *d_fq = nullptr;
    uint64_t fq_bytes = 0;
    int interleaved = 0;
    ParsedReads pr;
    // partition state
    uint32_t *d_parent = nullptr;
    uint32_t *d_size = nullptr;
    uint8_t *d_filtered = nullptr;
    // k-mer cache written by the count pass (plain variant), in pieces of consecutive reads (one piece,
    // or one per input segment of mp_job_load_count)
    int store = STORE_KMER_CACHE;  // what the count pass keeps of the reads for the partition (mp_job_set_read_store)
    int kc_k = 0;
    std::vector<KcPiece> kc;
    cudaStream_t copy_st = nullptr;  // uploads of mp_job_load_count
    int T = 0, nchunks = 0;
    std::vector<uint64_t> chunk_rec;
    uint64_t bounds[17] = {0};
    bool partitioned = false;
    // output
    uint8_t *d_out = nullptr;
    uint64_t out_total = 0;
    std::vector<uint64_t> out_sizes;
    bool output_ready = false;  // out_plan holds the partition files' layout
    OutputPlan out_plan;
    std::string dump_dir;
    double stage_ms[8] = {0};
    SortStats sort_stats;
    int sort_passes_total = 0;
    double sort_ms_total = 0;
    uint64_t sort_bytes_total = 0, sort_tuples_total = 0;
    double seg_ms_total = 0, big_ms_total = 0;
    uint64_t units_total = 0, big_buckets_total = 0, big_tuples_total = 0;
    uint64_t unit_passes_total = 0, phase_total[3] = {0, 0, 0}, pass_cycles_total[7] = {};
    int pe_rounds = 0;
    uint64_t piece_tuples = 0;  // most tuples a scan holds in HBM at once (0: from the free device memory)
    int pieces_total = 0;       // bucket-range pieces of the last partition, over all scans
    uint32_t hooked_bad = ~0u;  // a flagged read the last scan's unions hooked below a component (next scan: BAD)
    bool checks = false;        // self-checks of the sorted tuples and the final forest (mp_job_set_checks)
};

// ------------------------------------------------------------------ helpers

namespace {

int write_file(const std::string &path, const void *buf, size_t n, bool append = false)
{
    FILE *f = fopen(path.c_str(), append ? "ab" : "wb");
    if (!f) return set_error(MP_EIO, "cannot write %s", path.c_str());
    size_t w = n ? fwrite(buf, 1, n, f) : 0;
    fclose(f);
    if (w != n) return set_error(MP_EIO, "short write %s", path.c_str());
    return 0;
}

// Dump of tuples in the reference's 14-byte record format (enumerateKmers.c:352-365); append: after the
// file's earlier pieces.
int dump_tuples(mp_job *j, const char *name, const uint64_t *lo, const uint8_t *hi, const uint32_t *id, uint64_t n,
                bool append = false)
{
    if (j->dump_dir.empty()) return 0;
    const char *tu = getenv("MP_DUMP_TUPLES");  // "0": the per-read dumps only (large inputs)
    if (tu && strcmp(tu, "0") == 0) return 0;
    std::vector<uint64_t> hl(n);
    std::vector<uint8_t> hh(hi ? n : 0);
    std::vector<uint32_t> hid(n);
    if (n) {
        MP_CUDA(cudaMemcpyAsync(hl.data(), lo, n * 8, cudaMemcpyDeviceToHost, j->st));
        if (hi) MP_CUDA(cudaMemcpyAsync(hh.data(), hi, n, cudaMemcpyDeviceToHost, j->st));
        MP_CUDA(cudaMemcpyAsync(hid.data(), id, n * 4, cudaMemcpyDeviceToHost, j->st));
        MP_CUDA(cudaStreamSynchronize(j->st));
    }
    std::vector<uint8_t> b(n * 14);
    for (uint64_t i = 0; i < n; i++) {
        uint64_t kmer = (hl[i] >> 8) | (hi ? ((uint64_t)hh[i] << 56) : 0);
        uint16_t w4 = (uint16_t)(hl[i] & 0xFF);
        memcpy(&b[i * 14], &kmer, 8);
        memcpy(&b[i * 14 + 8], &w4, 2);
        memcpy(&b[i * 14 + 10], &hid[i], 4);
    }
    return write_file(j->dump_dir + "/" + name, b.data(), b.size(), append);
}

// Parent (5-byte encoding, BAD = 0xBADBADBAD) and sizes, as printStats leaves them.
int dump_state(mp_job *j, const char *pname, const char *sname, bool with_parent = true)
{
    if (j->dump_dir.empty()) return 0;
    const uint64_t n = j->pr.n_reads;
    std::vector<uint32_t> p(n), s(n);
    MP_CUDA(cudaMemcpyAsync(p.data(), j->d_parent, n * 4, cudaMemcpyDeviceToHost, j->st));
    MP_CUDA(cudaMemcpyAsync(s.data(), j->d_size, n * 4, cudaMemcpyDeviceToHost, j->st));
    MP_CUDA(cudaStreamSynchronize(j->st));
    int rc = 0;
    if (with_parent) {
        std::vector<uint8_t> b(n * 5);
        for (uint64_t i = 0; i < n; i++) {
            uint64_t v = p[i] == BAD ? 0xBADBADBADull : p[i];
            uint32_t rem = (uint32_t)(v % UMAX32);
            b[i * 5] = (uint8_t)(v / UMAX32);
            memcpy(&b[i * 5 + 1], &rem, 4);
        }
        rc = write_file(j->dump_dir + "/" + pname, b.data(), b.size());
    }
    if (!rc && sname) rc = write_file(j->dump_dir + "/" + sname, s.data(), n * 4);
    return rc;
}


__global__ void k_sizes_raw(const uint32_t *parent, uint64_t n, uint32_t *size)
{
    const uint64_t x = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const uint32_t p = parent[x];
    atomicAdd(&size[(p == BAD || p == x) ? (uint32_t)x : p], 1u);
}

// The reference's threshold walk over the prefix histogram (metapart.c:3728-3791):
//   for (i = 0; i < NB; i++) if (hist[i] >= step * cr) { record(cr, i); cr++; }
// hist is non-decreasing, so the cr-th hit is the later of the first bucket whose prefix reaches
// step * cr and the bucket after the previous hit: one binary search per hit instead of a pass over
// all buckets.  Hits after the maxc-th are not walked (the caller only tests the final counter
// against the last index).  Returns the final counter.
template <class F> static uint64_t threshold_walk(const uint64_t *hist, uint64_t step, uint64_t maxc, F record)
{
    uint64_t cr = 1;
    int64_t prev = -1;
    while (cr <= maxc) {
        const uint64_t lb = (uint64_t)(std::lower_bound(hist, hist + NB, step * cr) - hist);
        const uint64_t i = std::max<uint64_t>(lb, (uint64_t)(prev + 1));
        if (i >= NB) break;
        record(cr, i);
        prev = (int64_t)i;
        cr++;
    }
    return cr;
}

// The reference's scan / thread k-mer range planner at one rank (metapart.c:3720-3791).
int plan_ranges(const uint64_t *hist, int S, int T, std::vector<uint64_t> &scanR, std::vector<uint64_t> &thrR)
{
    const uint64_t total = hist[NB];
    if (total == 0) return set_error(MP_EUNSUP, "the histogram holds no k-mers");
    scanR.assign(S + 1, 0);
    thrR.assign((size_t)S * T + 1, 0);
    const uint64_t avg = total / (uint64_t)S + (total % (uint64_t)S ? 1 : 0);
    uint64_t cr = threshold_walk(hist, avg, (uint64_t)S, [&](uint64_t c, uint64_t i) { scanR[c] = i; });
    if (cr == (uint64_t)S) scanR[cr] = NB;
    const uint64_t avgT = avg / (uint64_t)T;
    cr = threshold_walk(hist, avgT, (uint64_t)S * T, [&](uint64_t c, uint64_t i) {
        thrR[c] = (c % (uint64_t)T == 0) ? scanR[c / T] : i;
    });
    if (cr == (uint64_t)S * T) thrR[cr] = NB;
    return 0;
}

// Tuple-index bounds of the thread ranges of one scan: the range partition bins a bucket
// to the last range whose start is not above it (metapart.c:2019-2022); the reference
// sizes its bins from [start_t, start_t+1) (metapart.c:1810-1850), so the two must agree.
// A bucket's bin is the largest t with max(ltr[0..t]) <= bucket, so bin t holds the buckets
// [M_t, M_t+1) with M_t the running maximum: each bin's count is one difference of the prefix.
int range_bounds(const uint64_t *hist, const uint64_t *ltr, int T, uint64_t scan_lo, uint64_t scan_hi,
                 std::vector<uint64_t> &bounds)
{
    if (scan_hi < scan_lo) scan_hi = scan_lo;  // an empty scan (the planner leaves trailing bounds at 0)
    auto clip = [&](uint64_t x) { return x < scan_lo ? scan_lo : (x > scan_hi ? scan_hi : x); };
    std::vector<uint64_t> M(T + 1);
    M[0] = ltr[0];
    for (int t = 1; t <= T; t++) M[t] = std::max(M[t - 1], ltr[t]);
    if (hist[clip(M[0])] != hist[scan_lo] || hist[scan_hi] != hist[clip(M[T])])
        return set_error(MP_EUNSUP, "thread k-mer ranges do not cover the scan's populated buckets");
    bounds.assign(T + 1, 0);
    for (int t = 0; t < T; t++) {
        const uint64_t c = hist[clip(M[t + 1])] - hist[clip(M[t])];
        const uint64_t ref = ltr[t + 1] > ltr[t] ? hist[ltr[t + 1]] - hist[ltr[t]] : 0;
        if (ref != c) return set_error(MP_EUNSUP, "thread k-mer ranges are not monotone over populated buckets");
        bounds[t + 1] = bounds[t] + c;
    }
    return 0;
}

void drop_kmer_cache(mp_job *j)
{
    for (KcPiece &q : j->kc) free_kc_piece(j->arena, q);
    j->kc.clear();
    j->kc_k = 0;
}

// The store of the reads for the plain variant's count pass (the job's choice: the k-mer cache or the packed
// reads), one piece for all reads; false (and no store) when the job keeps none or device memory or the
// budget does not allow it -- the partition then computes its k-mers from the FASTQ bytes.
bool make_kmer_cache(mp_job *j, int k)
{
    KcPiece q;
    const bool made = j->store == STORE_PACKED ? make_pk_piece(j->arena, j->st, j->pr, 0, k, &q)
                                               : make_kc_piece(j->arena, j->st, j->pr, 0, k, &q);
    if (!made) {
        drop_kmer_cache(j);
        return false;
    }
    j->kc.assign(1, q);
    j->kc_k = k;
    return true;
}

int chunk_records(mp_job *j, const uint64_t *chunk_starts, int nchunks, std::vector<uint64_t> &rec)
{
    rec.assign(nchunks + 1, 0);
    for (int c = 0; c < nchunks; c++)
        if (chunk_starts[c + 1] < chunk_starts[c]) return set_error(MP_EFMT, "chunk offsets are not ascending");
    if (chunk_starts[0] != 0 || chunk_starts[nchunks] != j->fq_bytes)
        return set_error(MP_EFMT, "chunks do not cover the input");
    return records_at_offsets(&j->pr, chunk_starts, nchunks + 1, rec.data(), j->arena, j->st);
}

}  // namespace

// ------------------------------------------------------------------ C ABI

extern "C" {

const char *mp_last_error(void) { return g_err.c_str(); }

int mp_ctx_create(int device, uint64_t hbm_budget_bytes, mp_ctx **out)
{
    if (!out) return set_error(MP_EARG, "null output pointer");
    int n = 0;
    MP_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return set_error(MP_EARG, "no CUDA device %d", device);
    MP_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    MP_CUDA(cudaGetDeviceProperties(&prop, device));
    if (prop.major < 10) return set_error(MP_EUNSUP, "device %d (%s) is not a Blackwell GPU", device, prop.name);
    mp_ctx *c = new mp_ctx;
    c->device = device;
    c->budget = hbm_budget_bytes ? hbm_budget_bytes : ~0ull;
    // keep freed stream-ordered memory in the pool between jobs
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    *out = c;
    return 0;
}

void mp_ctx_destroy(mp_ctx *ctx) { delete ctx; }

uint64_t mp_ctx_hbm_in_use(const mp_ctx *ctx) { return ctx ? ctx->used.load() : 0; }

int mp_job_create(mp_ctx *ctx, mp_job **out)
{
    if (!ctx || !out) return set_error(MP_EARG, "null argument");
    MP_CUDA(cudaSetDevice(ctx->device));
    mp_job *j = new mp_job;
    j->ctx = ctx;
    if (cudaStreamCreateWithFlags(&j->st, cudaStreamNonBlocking) != cudaSuccess) {
        delete j;
        return set_error(MP_ECUDA, "cannot create a stream");
    }
    j->arena.st = j->st;
    j->arena.budget_used = &ctx->used;
    j->arena.budget_limit = ctx->budget;
    const char *ck = getenv("MP_CHECK");
    j->checks = ck && *ck && *ck != '0';
    *out = j;
    return 0;
}

void mp_job_destroy(mp_job *job)
{
    if (!job) return;
    cudaSetDevice(job->ctx->device);
    job->arena.release_all();
    cudaStreamSynchronize(job->st);
    cudaStreamDestroy(job->st);
    if (job->copy_st) cudaStreamDestroy(job->copy_st);
    delete job;
}

static int load_common(mp_job *j, uint64_t nbytes, const uint64_t *file_sizes, int nfiles, int interleaved)
{
    uint64_t tot = 0;
    for (int f = 0; f < nfiles; f++) tot += file_sizes[f];
    if (tot != nbytes) return set_error(MP_EARG, "file sizes do not add up to the input size");
    j->fq_bytes = nbytes;
    j->interleaved = interleaved;
    j->stage_ms[0] = 0;
    {
        StageTimer tm(j->st, j->stage_ms, 0);
        int rc = parse_fastq(j->d_fq, nbytes, &j->pr, j->arena, j->st);
        if (rc) return rc;
    }
    // each file must end on a record end
    std::vector<uint64_t> ends;
    uint64_t acc = 0;
    for (int f = 0; f < nfiles; f++) { acc += file_sizes[f]; ends.push_back(acc); }
    ends.pop_back();
    if (!ends.empty()) {
        std::vector<uint64_t> rec(ends.size());
        int rc = records_at_offsets(&j->pr, ends.data(), (int)ends.size(), rec.data(), j->arena, j->st);
        if (rc) return set_error(MP_EFMT, "a FASTQ file does not end on a record boundary");
    }
    if (interleaved && (j->pr.n_reads & 1)) return set_error(MP_EFMT, "interleaved input with an odd record count");
    if (j->pr.n_reads >= UMAX32) return set_error(MP_EUNSUP, "more than 2^32 - 2 reads");
    return 0;
}

int mp_job_load_fastq(mp_job *j, const char *bytes, uint64_t nbytes, const uint64_t *file_sizes, int nfiles,
                      int interleaved)
{
    if (!j || !bytes || !file_sizes || nfiles < 1) return set_error(MP_EARG, "null argument");
    MP_CUDA(cudaSetDevice(j->ctx->device));
    if (j->d_fq) return set_error(MP_EARG, "the job already holds reads");
    j->d_fq = j->arena.alloc_persistent<uint8_t>(nbytes + 64);
    if (!j->d_fq) return set_error(MP_ENOMEM, "device memory for %llu FASTQ bytes", (unsigned long long)nbytes);
    MP_CUDA(cudaMemcpyAsync(j->d_fq, bytes, nbytes, cudaMemcpyHostToDevice, j->st));
    MP_CUDA(cudaMemsetAsync(j->d_fq + nbytes, 0, 64, j->st));
    return load_common(j, nbytes, file_sizes, nfiles, interleaved);
}

int mp_job_load_fastq_device(mp_job *j, const void *dev_bytes, uint64_t nbytes, const uint64_t *file_sizes, int nfiles,
                             int interleaved)
{
    if (!j || !dev_bytes || !file_sizes || nfiles < 1) return set_error(MP_EARG, "null argument");
    MP_CUDA(cudaSetDevice(j->ctx->device));
    if (j->d_fq) return set_error(MP_EARG, "the job already holds reads");
    j->d_fq = j->arena.alloc_persistent<uint8_t>(nbytes + 64);
    if (!j->d_fq) return set_error(MP_ENOMEM, "device memory for %llu FASTQ bytes", (unsigned long long)nbytes);
    MP_CUDA(cudaMemcpyAsync(j->d_fq, dev_bytes, nbytes, cudaMemcpyDeviceToDevice, j->st));
    MP_CUDA(cudaMemsetAsync(j->d_fq + nbytes, 0, 64, j->st));
    return load_common(j, nbytes, file_sizes, nfiles, interleaved);
}

int mp_job_load_fastq_device_inplace(mp_job *j, const void *dev_bytes, uint64_t nbytes, const uint64_t *file_sizes,
                                     int nfiles, int interleaved)
{
    if (!j || !dev_bytes || !file_sizes || nfiles < 1) return set_error(MP_EARG, "null argument");
    if ((uintptr_t)dev_bytes & 15) return set_error(MP_EARG, "the FASTQ bytes must start on a 16-byte boundary");
    MP_CUDA(cudaSetDevice(j->ctx->device));
    if (j->d_fq) return set_error(MP_EARG, "the job already holds reads");
    j->d_fq = (uint8_t *)dev_bytes;  // borrowed: not the arena's, so a reset drops it without freeing it
    return load_common(j, nbytes, file_sizes, nfiles, interleaved);
}

uint64_t mp_job_num_reads(const mp_job *j) { return j ? j->pr.n_reads : 0; }

int mp_job_reset(mp_job *j)
{
    if (!j) return set_error(MP_EARG, "null job");
    MP_CUDA(cudaSetDevice(j->ctx->device));
    j->arena.release_all();
    MP_CUDA(cudaStreamSynchronize(j->st));
    j->d_fq = nullptr;
    j->fq_bytes = 0;
    j->pr = ParsedReads{};
    j->d_parent = j->d_size = nullptr;
    j->d_filtered = nullptr;
    j->d_out = nullptr;
    j->out_plan = OutputPlan{};
    j->kc.clear();
    j->kc_k = 0;
    j->partitioned = j->output_ready = false;
    return 0;
}

void *mp_job_stream(mp_job *j) { return j ? (void *)j->st : nullptr; }

uint64_t mp_launch_count(void) { return g_launches.load(); }

int mp_job_count(mp_job *j, int k, int min3, const uint64_t *chunk_starts, int nchunks, uint64_t *hist_out,
                 uint32_t *chunk_counts_out, uint64_t *chunk_reads_out)
{
    if (!j || !j->d_fq || !chunk_starts || !hist_out || nchunks < 1) return set_error(MP_EARG, "bad argument");
    if (k < 11 || k > 31) return set_error(MP_EARG, "k must be in [11, 31]");
    MP_CUDA(cudaSetDevice(j->ctx->device));
    std::vector<uint64_t> rec;
    int rc = chunk_records(j, chunk_starts, nchunks, rec);
    if (rc) return rc;
    j->stage_ms[1] = 0;
    uint64_t *d_rec = j->arena.alloc<uint64_t>(nchunks + 1);
    unsigned long long *glob = j->arena.alloc<unsigned long long>(NB);
    uint32_t *cc = chunk_counts_out ? j->arena.alloc<uint32_t>((size_t)nchunks * NB) : nullptr;
    uint32_t *err = j->arena.alloc<uint32_t>(1);
    if (!d_rec || !glob || !err || (chunk_counts_out && !cc)) return set_error(MP_ENOMEM, "device memory for counting");
    MP_CUDA(cudaMemcpyAsync(d_rec, rec.data(), (nchunks + 1) * 8, cudaMemcpyHostToDevice, j->st));
    MP_CUDA(cudaMemsetAsync(glob, 0, NB * 8, j->st));
    MP_CUDA(cudaMemsetAsync(err, 0, 4, j->st));
    if (cc) MP_CUDA(cudaMemsetAsync(cc, 0, (size_t)nchunks * NB * 4, j->st));
    drop_kmer_cache(j);
    {
        StageTimer tm(j->st, j->stage_ms, 1);
        const bool kc = j->store != STORE_FASTQ && !min3 && make_kmer_cache(j, k);
        const KcPiece q = kc ? j->kc[0] : KcPiece{};
        launch_count(j->d_fq, j->pr, k, min3, d_rec, nchunks, cc, glob, err, j->st, q.off, q.lo, q.hi, q.poff, q.pw, q.pn);
    }
    std::vector<unsigned long long> g(NB);
    uint32_t herr = 0;
    MP_CUDA(cudaMemcpyAsync(g.data(), glob, NB * 8, cudaMemcpyDeviceToHost, j->st));
    MP_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, j->st));
    if (cc) MP_CUDA(cudaMemcpyAsync(chunk_counts_out, cc, (size_t)nchunks * NB * 4, cudaMemcpyDeviceToHost, j->st));
    MP_CUDA(cudaStreamSynchronize(j->st));
    MP_CUDA(cudaGetLastError());
    j->arena.release_scratch();
    if (herr & DERR_LONG_READ) {
        drop_kmer_cache(j);
        return set_error(MP_EUNSUP, "a read is longer than %d bases", MAX_READ_COUNT);
    }
    if (herr & DERR_NONACGT) drop_kmer_cache(j);  // a byte the packed reads cannot hold: the FASTQ path
    hist_out[0] = 0;
    for (uint32_t b = 1; b <= NB; b++) hist_out[b] = hist_out[b - 1] + g[b - 1];
    if (chunk_reads_out)
        for (int c = 0; c < nchunks; c++) chunk_reads_out[c] = rec[c + 1] - rec[c];
    return 0;
}

namespace {

constexpr int LC_SEGMENTS = 8;  // upload segments of mp_job_load_count

// The pipelined body of mp_job_load_count: segment i's bytes go up on the copy stream while the job
// stream parses and counts segment i - 1.  Each segment holds whole chunks, so it starts on a record
// start of the whole input exactly when its own parse succeeds (a segment whose lines are not a multiple
// of four, or that does not end with a complete record, fails); the segments' record tables then
// concatenate to the whole input's.  Any failure returns non-zero and the caller reruns the steps one
// after the other, which report it.
int load_count_pipelined(mp_job *j, const char *bytes, uint64_t nbytes, const uint64_t *file_sizes, int nfiles,
                         int interleaved, int k, const std::vector<uint64_t> &seg, const uint64_t *chunk_starts,
                         int nchunks, uint64_t *hist_out, uint64_t *chunk_reads_out)
{
    const int S = (int)seg.size() - 1;
    j->d_fq = j->arena.alloc_persistent<uint8_t>(nbytes + 64);
    if (!j->d_fq) return MP_ENOMEM;
    if (!j->copy_st && cudaStreamCreateWithFlags(&j->copy_st, cudaStreamNonBlocking) != cudaSuccess) {
        j->copy_st = nullptr;
        return MP_ECUDA;
    }
    std::vector<cudaEvent_t> ev(S + 1);
    for (auto &e : ev) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    struct Guard {  // the copies end before anything below returns (an error path frees the buffer)
        cudaStream_t cs;
        std::vector<cudaEvent_t> &ev;
        ~Guard()
        {
            cudaStreamSynchronize(cs);
            for (auto &e : ev) cudaEventDestroy(e);
        }
    } guard{j->copy_st, ev};
    cudaEventRecord(ev[S], j->st);  // the buffer exists
    cudaStreamWaitEvent(j->copy_st, ev[S], 0);
    for (int i = 0; i < S; i++) {
        if (cudaMemcpyAsync(j->d_fq + seg[i], bytes + seg[i], seg[i + 1] - seg[i], cudaMemcpyHostToDevice, j->copy_st) !=
            cudaSuccess)
            return MP_ECUDA;
        cudaEventRecord(ev[i], j->copy_st);
    }
    MP_CUDA(cudaMemsetAsync(j->d_fq + nbytes, 0, 64, j->st));
    uint64_t tot = 0;
    for (int f = 0; f < nfiles; f++) tot += file_sizes[f];
    if (tot != nbytes) return MP_EARG;
    j->fq_bytes = nbytes;
    j->interleaved = interleaved;
    j->stage_ms[0] = j->stage_ms[1] = 0;
    unsigned long long *glob = j->arena.alloc_persistent<unsigned long long>(NB);
    uint32_t *err = j->arena.alloc_persistent<uint32_t>(1);
    if (!glob || !err) return MP_ENOMEM;
    MP_CUDA(cudaMemsetAsync(glob, 0, NB * 8, j->st));
    MP_CUDA(cudaMemsetAsync(err, 0, 4, j->st));
    drop_kmer_cache(j);
    std::vector<ParsedReads> prs(S);
    std::vector<uint64_t> R(S + 1, 0);
    for (int i = 0; i < S; i++) {
        MP_CUDA(cudaStreamWaitEvent(j->st, ev[i], 0));
        {
            StageTimer tm(j->st, j->stage_ms, 0);
            if (parse_fastq_range(j->d_fq, seg[i], seg[i + 1], &prs[i], j->arena, j->st)) return MP_EFMT;
        }
        R[i + 1] = R[i] + prs[i].n_reads;
        StageTimer tm(j->st, j->stage_ms, 1);
        KcPiece q;
        const bool made = j->store == STORE_PACKED ? make_pk_piece(j->arena, j->st, prs[i], R[i], k, &q)
                                                   : make_kc_piece(j->arena, j->st, prs[i], R[i], k, &q);
        if (!made) return MP_ENOMEM;
        j->kc.push_back(q);
        launch_count(j->d_fq + seg[i], prs[i], k, 0, nullptr, 0, nullptr, glob, err, j->st, q.off, q.lo, q.hi, q.poff, q.pw,
                     q.pn);
    }
    j->kc_k = k;
    const uint64_t N = R[S];
    if (N >= UMAX32 || (interleaved && (N & 1))) return MP_EFMT;
    {
        StageTimer tm(j->st, j->stage_ms, 0);
        j->pr.n_reads = N;
        j->pr.rec_start = j->arena.alloc_persistent<uint64_t>(N + 1);
        j->pr.seq_off = j->arena.alloc_persistent<uint64_t>(N + 1);
        j->pr.seq_len = j->arena.alloc_persistent<uint32_t>(N + 1);
        if (!j->pr.rec_start || !j->pr.seq_off || !j->pr.seq_len) return MP_ENOMEM;
        for (int i = 0; i < S; i++) concat_records(prs[i], seg[i], j->pr, R[i], j->st);
    }
    for (auto &p : prs) {
        j->arena.free_persistent(p.rec_start);
        j->arena.free_persistent(p.seq_off);
        j->arena.free_persistent(p.seq_len);
    }
    // the checks of the load (files end on record ends) and of the count (chunks start on records)
    std::vector<uint64_t> ends;
    uint64_t acc = 0;
    for (int f = 0; f + 1 < nfiles; f++) ends.push_back(acc += file_sizes[f]);
    if (!ends.empty()) {
        std::vector<uint64_t> rec(ends.size());
        if (records_at_offsets(&j->pr, ends.data(), (int)ends.size(), rec.data(), j->arena, j->st)) return MP_EFMT;
    }
    std::vector<uint64_t> rec;
    if (chunk_records(j, chunk_starts, nchunks, rec)) return MP_EFMT;
    std::vector<unsigned long long> g(NB);
    uint32_t herr = 0;
    MP_CUDA(cudaMemcpyAsync(g.data(), glob, NB * 8, cudaMemcpyDeviceToHost, j->st));
    MP_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, j->st));
    MP_CUDA(cudaStreamSynchronize(j->st));
    MP_CUDA(cudaGetLastError());
    j->arena.free_persistent(glob);
    j->arena.free_persistent(err);
    j->arena.release_scratch();
    if (herr & DERR_NONACGT) drop_kmer_cache(j);  // a byte the packed reads cannot hold: the FASTQ path
    if (herr & ~DERR_NONACGT) return MP_EUNSUP;
    hist_out[0] = 0;
    for (uint32_t b = 1; b <= NB; b++) hist_out[b] = hist_out[b - 1] + g[b - 1];
    if (chunk_reads_out)
        for (int c = 0; c < nchunks; c++) chunk_reads_out[c] = rec[c + 1] - rec[c];
    return 0;
}

}  // namespace

int mp_job_load_count(mp_job *j, const char *bytes, uint64_t nbytes, const uint64_t *file_sizes, int nfiles,
                      int interleaved, int k, int min3, const uint64_t *chunk_starts, int nchunks, uint64_t *hist_out,
                      uint64_t *chunk_reads_out)
{
    if (!j || !bytes || !file_sizes || nfiles < 1 || !chunk_starts || !hist_out || nchunks < 1)
        return set_error(MP_EARG, "bad argument");
    if (k < 11 || k > 31) return set_error(MP_EARG, "k must be in [11, 31]");
    MP_CUDA(cudaSetDevice(j->ctx->device));
    if (j->d_fq) return set_error(MP_EARG, "the job already holds reads");
    auto one_by_one = [&]() -> int {
        int rc = mp_job_load_fastq(j, bytes, nbytes, file_sizes, nfiles, interleaved);
        return rc ? rc : mp_job_count(j, k, min3, chunk_starts, nchunks, hist_out, nullptr, chunk_reads_out);
    };
    // pinned input (asynchronous copies), the k-mer cache variant, ascending chunks over the whole input
    cudaPointerAttributes pa{};
    const bool pinned = cudaPointerGetAttributes(&pa, bytes) == cudaSuccess && pa.type == cudaMemoryTypeHost;
    cudaGetLastError();
    bool ok = pinned && !min3 && j->store != STORE_FASTQ && nchunks >= 2 && chunk_starts[0] == 0 &&
              chunk_starts[nchunks] == nbytes;
    for (int c = 0; ok && c < nchunks; c++) ok = chunk_starts[c] <= chunk_starts[c + 1];
    if (!ok) return one_by_one();
    std::vector<uint64_t> seg = {0};
    for (int c = 1; c < nchunks; c++)
        if (chunk_starts[c] > seg.back() && chunk_starts[c] >= (uint64_t)((double)nbytes * seg.size() / LC_SEGMENTS))
            seg.push_back(chunk_starts[c]);
    seg.push_back(nbytes);
    if (seg.size() < 3) return one_by_one();
    if (load_count_pipelined(j, bytes, nbytes, file_sizes, nfiles, interleaved, k, seg, chunk_starts, nchunks, hist_out,
                             chunk_reads_out) == 0)
        return 0;
    int rc = mp_job_reset(j);
    return rc ? rc : one_by_one();
}

static void add_sort_stats(mp_job *j, const SortStats &ss, uint64_t n)
{
    j->sort_stats = ss;
    j->sort_passes_total += ss.passes;
    j->sort_ms_total += ss.pass_ms;
    j->sort_bytes_total += ss.bytes;
    j->sort_tuples_total += n;
    j->seg_ms_total += ss.seg_ms;
    j->big_ms_total += ss.big_ms;
    j->units_total += ss.units;
    j->big_buckets_total += ss.big_buckets;
    j->big_tuples_total += ss.big_tuples;
    j->unit_passes_total += ss.unit_passes;
    for (int q = 0; q < 3; q++) j->phase_total[q] += ss.phase_cycles[q];
    for (int q = 0; q < 7; q++) j->pass_cycles_total[q] += ss.pass_cycles[q];
}

// Most tuples one scan may hold in HBM at once: MP_SCAN_PIECE_TUPLES, else the job's setting, else what
// the context's budget (or the device, counting the pool's cached memory) has left at ~32 B per tuple
// (two tuple buffers of 13 B, the sort's status and plans, the filter's marks).
static uint64_t scan_piece_cap(mp_job *j)
{
    const char *e = getenv("MP_SCAN_PIECE_TUPLES");
    if (e && *e) return std::max<uint64_t>(1, strtoull(e, nullptr, 10));
    if (j->piece_tuples) return j->piece_tuples;
    size_t fr = 0, tot = 0;
    uint64_t avail = cudaMemGetInfo(&fr, &tot) == cudaSuccess ? fr : 0;
    cudaMemPool_t pool;
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t rsv = 0, used = 0;
        if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &rsv) == cudaSuccess &&
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && rsv > used)
            avail += rsv - used;
    }
    cudaGetLastError();
    if (j->arena.budget_used && j->arena.budget_limit != ~0ull) {
        const uint64_t u = j->arena.budget_used->load();
        avail = std::min<uint64_t>(avail, u < j->arena.budget_limit ? j->arena.budget_limit - u : 0);
    }
    return std::max<uint64_t>(1, avail / 32);
}

// Bucket-range pieces of the scan [lo, hi): consecutive buckets while their tuples stay within cap (a bucket
// above cap ends a piece of its own, with the empty buckets before it).  Returns the piece bounds, lo first
// and hi last.
static std::vector<uint64_t> plan_pieces(const uint64_t *hist, uint64_t lo, uint64_t hi, uint64_t cap)
{
    std::vector<uint64_t> b{lo};
    uint64_t start = lo;
    for (uint64_t x = lo + 1; x < hi; x++)
        if (hist[x + 1] - hist[start] > cap && hist[x] > hist[start]) {
            b.push_back(x);
            start = x;
        }
    b.push_back(hi);
    return b;
}

// One scan whose tuples do not fit HBM at once, in bucket-range pieces (the sorted scan is the pieces'
// sorted tuples one after the other).  Inside a scan every BAD mark is final before the first union
// (metapart.c:3961-3964), so the pieces are swept twice: enumerate, sort and filter each (its zero marks
// kept), then enumerate and sort each again and run its unions.  The enumeration of scans after the first
// carries each read's root as the scan began (SCAN_OPT, metapart.c:543-568), from a copy of the parents
// taken before the first sweep.  A thread range's last run is exempt from the filter only where the range
// ends, and each range's sweep starts from the scan's own initial state (metapart.c:2539-2548), however
// the pieces cut it.
// The sort self-check (mp_job_set_checks): no adjacent tuple pair out of (k-mer, adjacency) order.
static int check_sorted(mp_job *j, const uint64_t *lo, const uint8_t *hi, uint64_t n, int scan)
{
    if (!j->checks) return 0;
    unsigned long long *dc = j->arena.alloc<unsigned long long>(1);
    if (!dc) return set_error(MP_ENOMEM, "device memory");
    uint64_t bad = 0;
    int rc = count_unsorted(lo, hi, n, dc, j->st, &bad);
    j->arena.free_scratch(dc);
    if (rc) return rc;
    if (bad)
        return set_error(MP_EDEVICE, "check: scan %d's sorted tuples hold %llu adjacent pairs out of order", scan,
                         (unsigned long long)bad);
    return 0;
}

static int scan_in_pieces(mp_job *j, int s, int k, bool has_hi, uint64_t lo, uint64_t hi, const std::vector<uint64_t> &pcs,
                          const std::vector<uint64_t> &rb, const uint64_t *hist, const uint64_t *d_hist, bool use_kc,
                          uint32_t *err)
{
    const uint64_t N = j->pr.n_reads, scan0 = hist[lo];
    const int P = (int)pcs.size() - 1, T = (int)rb.size() - 1;
    int rc = 0;
    char name[64];
    uint64_t maxn = 0;
    for (int i = 0; i < P; i++) maxn = std::max<uint64_t>(maxn, hist[pcs[i + 1]] - hist[pcs[i]]);
    uint32_t *roots = nullptr;
    if (s) {
        roots = j->arena.alloc<uint32_t>(N + 1);
        if (!roots) return set_error(MP_ENOMEM, "device memory for the scan's roots");
        MP_CUDA(cudaMemcpyAsync(roots, j->d_parent, (N + 1) * 4, cudaMemcpyDeviceToDevice, j->st));
    }
    uint32_t *cnt = j->arena.alloc<uint32_t>(N + 1), *d_b = j->arena.alloc<uint32_t>(2 * P);
    uint64_t *off = j->arena.alloc<uint64_t>(N + 2), *ntot = j->arena.alloc<uint64_t>(1);
    const size_t tb = scan_tmp_bytes(N + 1);
    void *tmp = j->arena.alloc<uint8_t>(tb);
    SortBufs sb0;
    for (int b = 0; b < 2; b++) {
        sb0.lo[b] = j->arena.alloc<uint64_t>(maxn + 1);
        sb0.id[b] = j->arena.alloc<uint32_t>(maxn + 1);
        sb0.hi[b] = has_hi ? j->arena.alloc<uint8_t>(maxn + 1) : nullptr;
        if (!sb0.lo[b] || !sb0.id[b] || (has_hi && !sb0.hi[b]))
            return set_error(MP_ENOMEM, "device memory for %llu tuples", (unsigned long long)maxn);
    }
    if (!cnt || !d_b || !off || !ntot || !tmp) return set_error(MP_ENOMEM, "device memory for enumeration offsets");
    {
        std::vector<uint32_t> hb(2 * P);
        for (int i = 0; i < P; i++) hb[2 * i] = (uint32_t)pcs[i], hb[2 * i + 1] = (uint32_t)pcs[i + 1];
        MP_CUDA(cudaMemcpyAsync(d_b, hb.data(), hb.size() * 4, cudaMemcpyHostToDevice, j->st));
    }
    // piece i's tuples in enumeration order into sb0.*[0], then sorted; tp views the sorted piece
    auto piece_tuples = [&](int i, Tuples &tp) -> int {
        const uint64_t b0 = pcs[i], b1 = pcs[i + 1], expect = hist[b1] - hist[b0];
        SortBufs sb = sb0;
        uint64_t n = 0;
        {
            StageTimer tm(j->st, j->stage_ms, 2);
            int lrc = 0;
            if (use_kc)
                for (const KcPiece &q : j->kc) lrc |= store_count_scans(q, j->pr.seq_len, k, d_b + 2 * i, 1, cnt, N + 1, err, j->st);
            else
                launch_enum_count(j->d_fq, j->pr, k, 0, (uint32_t)b0, (uint32_t)b1, cnt, err, j->st);
            if (lrc) return set_error(MP_EARG, "enumeration count of a scan piece");
            MP_CUDA(cudaMemsetAsync(cnt + N, 0, 4, j->st));
            scan_u32_to_u64(cnt, off, N + 1, ntot, tmp, tb, j->st);
            MP_CUDA(cudaMemcpyAsync(&n, ntot, 8, cudaMemcpyDeviceToHost, j->st));
            MP_CUDA(cudaStreamSynchronize(j->st));
            if (n != expect)
                return set_error(MP_EFMT, "scan %d piece %d: %llu tuples but the histogram holds %llu", s, i,
                                 (unsigned long long)n, (unsigned long long)expect);
            if (use_kc)
                for (const KcPiece &q : j->kc)
                    store_write(q, j->pr.seq_len, k, (uint32_t)b0, (uint32_t)b1, roots, off, sb.lo[0], sb.hi[0], sb.id[0], err,
                                j->st);
            else
                launch_enum_write(j->d_fq, j->pr, k, 0, (uint32_t)b0, (uint32_t)b1, roots, off, sb.lo[0], sb.hi[0],
                                  sb.id[0], err, j->st);
        }
        uint32_t herr = 0;
        MP_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, j->st));
        MP_CUDA(cudaStreamSynchronize(j->st));
        if (herr) return set_error(MP_EDEVICE, "enumeration flags 0x%x", herr);
        int lo_buf = 0, hi_buf = 0;
        {
            StageTimer tm(j->st, j->stage_ms, 3);
            SortStats ss;
            int r = bucket_sort(sb, n, has_hi, k, d_hist, b0, b1, j->arena, j->st, &ss, &lo_buf, &hi_buf);
            if (r) return r;
            add_sort_stats(j, ss, n);
        }
        tp = Tuples{};
        tp.lo = sb.lo[lo_buf];
        tp.hi = has_hi ? sb.hi[hi_buf] : nullptr;
        tp.id = sb.id[lo_buf];
        tp.n = n;
        return 0;
    };
    // ---- sweep 1: the filter over every piece
    std::vector<uint32_t *> zs(P);
    uint32_t first_id = 0;
    uint64_t last_kmer = 0;
    bool have_first = false;
    for (int i = 0; i < P; i++) {
        Tuples tp;
        if ((rc = piece_tuples(i, tp))) return rc;
        const uint64_t p0 = hist[pcs[i]] - scan0, p1 = hist[pcs[i + 1]] - scan0;
        if ((rc = check_sorted(j, tp.lo, tp.hi, tp.n, s))) return rc;
        snprintf(name, sizeof name, "scan%d_sorted.bin", s);
        if ((rc = dump_tuples(j, name, tp.lo, tp.hi, tp.id, tp.n, i > 0))) return rc;
        std::vector<uint64_t> ends{0};  // the thread ranges ending inside the piece or at its end
        for (int t = 1; t <= T; t++)
            if (rb[t] > p0 && rb[t] <= p1) ends.push_back(rb[t] - p0);
        {
            StageTimer tm(j->st, j->stage_ms, 4);
            if ((rc = filter_scan(tp, ends, j->d_parent, j->d_filtered, j->arena, j->st, !j->dump_dir.empty()))) return rc;
        }
        zs[i] = tp.z;
        snprintf(name, sizeof name, "scan%d_filtered.bin", s);
        if ((rc = dump_tuples(j, name, tp.lo, tp.hi, tp.id, tp.n, i > 0))) return rc;
        if (tp.n && !have_first) {  // the scan's first tuple
            MP_CUDA(cudaMemcpyAsync(&first_id, tp.id, 4, cudaMemcpyDeviceToHost, j->st));
            have_first = true;
        }
        if (tp.n) {  // the scan's last tuple, once the last piece that holds one is done
            uint64_t l = 0;
            uint8_t h = 0;
            uint32_t zw = 0;
            MP_CUDA(cudaMemcpyAsync(&l, tp.lo + (tp.n - 1), 8, cudaMemcpyDeviceToHost, j->st));
            if (tp.hi) MP_CUDA(cudaMemcpyAsync(&h, tp.hi + (tp.n - 1), 1, cudaMemcpyDeviceToHost, j->st));
            MP_CUDA(cudaMemcpyAsync(&zw, tp.z + ((tp.n - 1) >> 5), 4, cudaMemcpyDeviceToHost, j->st));
            MP_CUDA(cudaStreamSynchronize(j->st));
            last_kmer = ((zw >> ((tp.n - 1) & 31)) & 1u) ? 0 : ((l >> 8) | ((uint64_t)h << 56));
        }
        MP_CUDA(cudaStreamSynchronize(j->st));
    }
    if (!j->dump_dir.empty()) {
        std::vector<uint8_t> f(N);
        MP_CUDA(cudaMemcpyAsync(f.data(), j->d_filtered, N, cudaMemcpyDeviceToHost, j->st));
        MP_CUDA(cudaStreamSynchronize(j->st));
        snprintf(name, sizeof name, "scan%d_bad.bin", s);
        rc = write_file(j->dump_dir + "/" + name, f.data(), N);
        if (rc) return rc;
    }
    // ---- sweep 2: the unions, piece by piece, from the scan's initial state
    rebad_read(j->d_parent, j->hooked_bad, j->st);
    j->hooked_bad = ~0u;
    uint32_t *anchor = j->arena.alloc<uint32_t>(2);  // the anchor run's read, the hooked read
    if (!anchor) return set_error(MP_ENOMEM, "device memory");
    MP_CUDA(cudaMemsetAsync(anchor, 0xFF, 8, j->st));
    uint32_t first_parent = 0;
    MP_CUDA(cudaMemcpyAsync(&first_parent, j->d_parent + first_id, 4, cudaMemcpyDeviceToHost, j->st));
    MP_CUDA(cudaStreamSynchronize(j->st));
    std::vector<uint8_t> seen(T, 0);
    for (int i = 0; i < P; i++) {
        Tuples tp;
        if ((rc = piece_tuples(i, tp))) return rc;
        tp.z = zs[i];
        const uint64_t p0 = hist[pcs[i]] - scan0, p1 = hist[pcs[i + 1]] - scan0;
        std::vector<uint64_t> bounds;  // the piece's parts of the thread ranges, and which range each is
        std::vector<int> which;
        for (int t = 0; t < T; t++) {
            const uint64_t a = std::max(rb[t], p0), b = std::min(rb[t + 1], p1);
            if (a < b) {
                bounds.push_back(a - p0);
                which.push_back(t);
            }
        }
        bounds.push_back(p1 - p0);
        std::vector<uint8_t> part_seen(which.size()), has_valid;
        for (size_t q = 0; q < which.size(); q++) part_seen[q] = seen[which[q]];
        {
            StageTimer tm(j->st, j->stage_ms, 5);
            if ((rc = union_piece(tp, bounds, part_seen, last_kmer, first_id, first_parent != BAD, j->d_parent,
                                  j->d_filtered, j->arena, j->st, has_valid, anchor)))
                return rc;
        }
        for (size_t q = 0; q < which.size(); q++) seen[which[q]] |= has_valid[q];
    }
    {
        StageTimer tm(j->st, j->stage_ms, 5);
        if (have_first && first_parent == BAD) hook_bad_anchor(j->d_parent, first_id, anchor, anchor + 1, j->st);
        compress_parents(j->d_parent, N, j->st);
        MP_CUDA(cudaMemcpyAsync(&j->hooked_bad, anchor + 1, 4, cudaMemcpyDeviceToHost, j->st));
        MP_CUDA(cudaStreamSynchronize(j->st));
        MP_CUDA(cudaGetLastError());
    }
    j->pieces_total += P;
    return 0;
}

int mp_job_partition(mp_job *j, const mp_part_params *p, const uint64_t *chunk_starts, const uint64_t *chunk_first_read,
                     int nchunks, const uint64_t *hist, uint64_t *bounds_out)
{
    if (!j || !j->d_fq || !p || !chunk_starts || !chunk_first_read || !hist || nchunks < 1)
        return set_error(MP_EARG, "bad argument");
    const int k = p->k, S = p->num_scans, T = p->num_threads;
    if (k < 11 || k > 31) return set_error(MP_EARG, "k must be in [11, 31]");
    if (S < 1 || T < 1 || T > 256) return set_error(MP_EARG, "numScans must be >= 1 and numThreads in [1, 256]");
    if (nchunks % T) return set_error(MP_EARG, "numThreads must divide the number of chunks");
    if (p->min3 && S != 1) return set_error(MP_EUNSUP, "the 3-minimizer variant needs numScans == 1");
    MP_CUDA(cudaSetDevice(j->ctx->device));
    const uint64_t N = j->pr.n_reads;
    std::vector<uint64_t> rec;
    int rc = chunk_records(j, chunk_starts, nchunks, rec);
    if (rc) return rc;
    for (int c = 0; c <= nchunks; c++)
        if (chunk_first_read[c] != rec[c])
            return set_error(MP_EFMT, "index read id of chunk %d (%llu) does not match the FASTQ (%llu)", c,
                             (unsigned long long)chunk_first_read[c], (unsigned long long)rec[c]);
    if (N & 1) return set_error(MP_EUNSUP, "the mate union needs an even read count");
    if (j->interleaved)
        for (int c = 0; c < nchunks; c++)
            if ((rec[c + 1] - rec[c]) & 1) return set_error(MP_EFMT, "interleaved chunk %d has an odd record count", c);
    std::vector<uint64_t> scanR, thrR;
    if ((rc = plan_ranges(hist, S, T, scanR, thrR))) return rc;
    j->T = T;
    j->nchunks = nchunks;
    j->chunk_rec = rec;
    j->partitioned = false;
    j->output_ready = false;
    for (int s = 2; s < 8; s++) j->stage_ms[s] = 0;
    j->sort_passes_total = 0;
    j->sort_ms_total = 0;
    j->sort_bytes_total = 0;
    j->sort_tuples_total = 0;
    j->seg_ms_total = 0;
    j->big_ms_total = 0;
    j->units_total = j->big_buckets_total = j->big_tuples_total = 0;
    j->unit_passes_total = 0;
    for (auto &v : j->phase_total) v = 0;
    for (auto &v : j->pass_cycles_total) v = 0;
    if (j->d_parent) { j->arena.free_persistent(j->d_parent); j->d_parent = nullptr; }
    if (j->d_size) { j->arena.free_persistent(j->d_size); j->d_size = nullptr; }
    if (j->d_filtered) { j->arena.free_persistent(j->d_filtered); j->d_filtered = nullptr; }
    if (j->d_out) { j->arena.free_persistent(j->d_out); j->d_out = nullptr; }
    j->arena.free_persistent(j->out_plan.val);
    j->arena.free_persistent(j->out_plan.off);
    j->out_plan = OutputPlan{};
    j->d_parent = j->arena.alloc_persistent<uint32_t>(N + 1);
    j->d_size = j->arena.alloc_persistent<uint32_t>(N + 1);
    j->d_filtered = j->arena.alloc_persistent<uint8_t>(N + 1);
    uint32_t *err = j->arena.alloc_persistent<uint32_t>(1);
    if (!j->d_parent || !j->d_size || !j->d_filtered || !err) return set_error(MP_ENOMEM, "device memory for the forest");
    const unsigned gN = (unsigned)((N + 255) / 256);
    launch_init_parent(j->d_parent, N, j->st);
    MP_CUDA(cudaMemsetAsync(j->d_filtered, 0, N + 1, j->st));
    MP_CUDA(cudaMemsetAsync(err, 0, 4, j->st));
    const bool has_hi = 2 * k + 8 > 64;
    char name[64], name2[64];
    // tuples per read of every scan in one pass (plain variant, monotone scan bounds)
    // the histogram prefix on the device, for the sort's planning kernels
    uint64_t *d_hist = j->arena.alloc_persistent<uint64_t>(NB + 1);
    if (!d_hist) return set_error(MP_ENOMEM, "device memory for the histogram");
    MP_CUDA(cudaMemcpyAsync(d_hist, hist, (NB + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, j->st));
    uint32_t *cnt_all = nullptr, *d_b = nullptr;
    // the count pass's k-mer cache serves this partition when it holds the same k (plain variant)
    const bool use_kc = !j->kc.empty() && j->kc_k == k && !p->min3 && S <= 8;
    {
        bool mono = !p->min3 && S <= 8;
        for (int s = 0; s < S && mono; s++) mono = scanR[s] <= scanR[s + 1];
        if (mono) {
            cnt_all = j->arena.alloc_persistent<uint32_t>((size_t)S * (N + 1));
            d_b = j->arena.alloc_persistent<uint32_t>(S + 1);
            if (!cnt_all || !d_b) return set_error(MP_ENOMEM, "device memory for enumeration counts");
            std::vector<uint32_t> hb(scanR.begin(), scanR.end());
            StageTimer tm(j->st, j->stage_ms, 2);
            MP_CUDA(cudaMemcpyAsync(d_b, hb.data(), (S + 1) * 4, cudaMemcpyHostToDevice, j->st));
            int lrc = 0;
            if (use_kc)
                for (const KcPiece &q : j->kc) lrc |= store_count_scans(q, j->pr.seq_len, k, d_b, S, cnt_all, N + 1, err, j->st);
            else
                lrc = launch_enum_count_scans(j->d_fq, j->pr, k, d_b, S, cnt_all, N + 1, err, j->st);
            if (lrc) return set_error(MP_EARG, "enumeration count over %d scans", S);
            for (int s = 0; s < S; s++) MP_CUDA(cudaMemsetAsync(cnt_all + (size_t)s * (N + 1) + N, 0, 4, j->st));
        }
    }
    j->pieces_total = 0;
    j->hooked_bad = ~0u;
    const uint64_t piece_cap = p->min3 ? ~0ull : scan_piece_cap(j);  // the 3-minimizer choice depends on the range
    for (int s = 0; s < S; s++) {
        const uint64_t lo = scanR[s], hi = scanR[s + 1];
        const uint64_t expect = hist[hi] - hist[lo];
        if (expect > piece_cap) {
            const std::vector<uint64_t> pcs = plan_pieces(hist, lo, hi, piece_cap);
            if (pcs.size() > 2) {
                {  // the per-read checks of the whole scan (its counts, when the pass over all scans did not make them)
                    uint32_t cerr = 0, *c1 = cnt_all ? nullptr : j->arena.alloc<uint32_t>(N + 1);
                    if (!cnt_all && !c1) return set_error(MP_ENOMEM, "device memory for enumeration counts");
                    if (c1) launch_enum_count(j->d_fq, j->pr, k, 0, (uint32_t)lo, (uint32_t)hi, c1, err, j->st);
                    MP_CUDA(cudaMemcpyAsync(&cerr, err, 4, cudaMemcpyDeviceToHost, j->st));
                    MP_CUDA(cudaStreamSynchronize(j->st));
                    j->arena.free_scratch(c1);
                    if (cerr & DERR_LONG_READ) return set_error(MP_EUNSUP, "a read has 300 or more k-mer positions");
                    if (cerr & DERR_TOO_MANY)
                        return set_error(MP_EUNSUP, "a read has 256 or more k-mers in scan %d (the reference counts "
                                                    "them in 8 bits, enumerateKmers.c:152)", s);
                    if (cerr) return set_error(MP_EDEVICE, "enumeration flags 0x%x", cerr);
                }
                std::vector<uint64_t> rb;
                if ((rc = range_bounds(hist, thrR.data() + (size_t)s * T, T, lo, hi, rb))) return rc;
                if ((rc = scan_in_pieces(j, s, k, has_hi, lo, hi, pcs, rb, hist, d_hist, use_kc, err))) return rc;
                j->arena.release_scratch();
                snprintf(name, sizeof name, "stats%d_parent.bin", s);
                if ((rc = dump_state(j, name, nullptr))) return rc;
                continue;
            }
        }
        j->pieces_total += 1;
        uint32_t *cnt = cnt_all ? cnt_all + (size_t)s * (N + 1) : j->arena.alloc<uint32_t>(N + 1);
        uint64_t *off = j->arena.alloc<uint64_t>(N + 2), *ntot = j->arena.alloc<uint64_t>(1);
        size_t tb = scan_tmp_bytes(N + 1);
        void *tmp = j->arena.alloc<uint8_t>(tb);
        if (!cnt || !off || !ntot || !tmp) return set_error(MP_ENOMEM, "device memory for enumeration offsets");
        SortBufs sb;
        int lo_buf = 0, hi_buf = 0;
        uint64_t n = 0;
        {
            StageTimer tm(j->st, j->stage_ms, 2);
            if (!cnt_all) {
                launch_enum_count(j->d_fq, j->pr, k, p->min3, (uint32_t)lo, (uint32_t)hi, cnt, err, j->st);
                MP_CUDA(cudaMemsetAsync(cnt + N, 0, 4, j->st));
            }
            scan_u32_to_u64(cnt, off, N + 1, ntot, tmp, tb, j->st);
            uint32_t cerr = 0;
            MP_CUDA(cudaMemcpyAsync(&n, ntot, 8, cudaMemcpyDeviceToHost, j->st));
            MP_CUDA(cudaMemcpyAsync(&cerr, err, 4, cudaMemcpyDeviceToHost, j->st));
            MP_CUDA(cudaStreamSynchronize(j->st));
            if (cerr & DERR_LONG_READ) return set_error(MP_EUNSUP, "a read has 300 or more k-mer positions");
            if (cerr & DERR_TOO_MANY)
                return set_error(MP_EUNSUP, "a read has 256 or more k-mers in scan %d (the reference counts them "
                                            "in 8 bits, enumerateKmers.c:152)", s);
            if (n != expect)
                return set_error(MP_EFMT, "scan %d: %llu tuples but the histogram holds %llu", s, (unsigned long long)n,
                                 (unsigned long long)expect);
            for (int b = 0; b < 2; b++) {
                sb.lo[b] = j->arena.alloc<uint64_t>(n + 1);
                sb.id[b] = j->arena.alloc<uint32_t>(n + 1);
                sb.hi[b] = has_hi ? j->arena.alloc<uint8_t>(n + 1) : nullptr;
                if (!sb.lo[b] || !sb.id[b] || (has_hi && !sb.hi[b]))
                    return set_error(MP_ENOMEM, "device memory for %llu tuples", (unsigned long long)n);
            }
            if (use_kc && cnt_all)
                for (const KcPiece &q : j->kc)
                    store_write(q, j->pr.seq_len, k, (uint32_t)lo, (uint32_t)hi, s ? j->d_parent : nullptr, off, sb.lo[0],
                                sb.hi[0], sb.id[0], err, j->st);
            else
                launch_enum_write(j->d_fq, j->pr, k, p->min3, (uint32_t)lo, (uint32_t)hi, s ? j->d_parent : nullptr, off,
                                  sb.lo[0], sb.hi[0], sb.id[0], err, j->st);
        }
        uint32_t herr = 0;
        MP_CUDA(cudaMemcpyAsync(&herr, err, 4, cudaMemcpyDeviceToHost, j->st));
        MP_CUDA(cudaStreamSynchronize(j->st));
        if (herr & DERR_LONG_READ) return set_error(MP_EUNSUP, "a read has 300 or more k-mer positions");
        if (herr & DERR_TOO_MANY)
            return set_error(MP_EUNSUP, "a read has 256 or more k-mers in scan %d (the reference counts them in 8 bits, "
                                        "enumerateKmers.c:152)", s);
        if (herr) return set_error(MP_EDEVICE, "enumeration flags 0x%x", herr);
        snprintf(name, sizeof name, "scan%d_enum.bin", s);
        if ((rc = dump_tuples(j, name, sb.lo[0], sb.hi[0], sb.id[0], n))) return rc;
        {
            StageTimer tm(j->st, j->stage_ms, 3);
            SortStats ss;
            if ((rc = bucket_sort(sb, n, has_hi, k, d_hist, lo, hi, j->arena, j->st, &ss, &lo_buf, &hi_buf))) return rc;
            add_sort_stats(j, ss, n);
        }
        Tuples tp;
        tp.lo = sb.lo[lo_buf];
        tp.hi = has_hi ? sb.hi[hi_buf] : nullptr;
        tp.id = sb.id[lo_buf];
        tp.n = n;
        if ((rc = check_sorted(j, tp.lo, tp.hi, n, s))) return rc;
        snprintf(name, sizeof name, "scan%d_sorted.bin", s);
        if ((rc = dump_tuples(j, name, tp.lo, tp.hi, tp.id, n))) return rc;
        std::vector<uint64_t> rb;
        if ((rc = range_bounds(hist, thrR.data() + (size_t)s * T, T, lo, hi, rb))) return rc;
        {
            StageTimer tm(j->st, j->stage_ms, 4);
            if ((rc = filter_scan(tp, rb, j->d_parent, j->d_filtered, j->arena, j->st, !j->dump_dir.empty()))) return rc;
        }
        snprintf(name, sizeof name, "scan%d_filtered.bin", s);
        if ((rc = dump_tuples(j, name, tp.lo, tp.hi, tp.id, n))) return rc;
        if (!j->dump_dir.empty()) {
            std::vector<uint8_t> f(N);
            MP_CUDA(cudaMemcpyAsync(f.data(), j->d_filtered, N, cudaMemcpyDeviceToHost, j->st));
            MP_CUDA(cudaStreamSynchronize(j->st));
            snprintf(name, sizeof name, "scan%d_bad.bin", s);
            rc = write_file(j->dump_dir + "/" + name, f.data(), N);
            if (rc) return rc;
        }
        {
            StageTimer tm(j->st, j->stage_ms, 5);
            if ((rc = union_scan(tp, rb, j->d_parent, j->d_filtered, N, j->arena, j->st, j->hooked_bad, &j->hooked_bad)))
                return rc;
        }
        j->arena.release_scratch();
        snprintf(name, sizeof name, "stats%d_parent.bin", s);
        if ((rc = dump_state(j, name, nullptr))) return rc;
    }
    j->arena.free_persistent(cnt_all);
    j->arena.free_persistent(d_b);
    j->arena.free_persistent(d_hist);
    drop_kmer_cache(j);  // its HBM goes back before the mate union and the output
    {
        StageTimer tm(j->st, j->stage_ms, 6);
        if (!j->dump_dir.empty()) {
            MP_CUDA(cudaMemsetAsync(j->d_size, 0, N * 4, j->st));
            (mp::count_launch(), k_sizes_raw<<<gN, 256, 0, j->st>>>(j->d_parent, N, j->d_size));
            snprintf(name, sizeof name, "stats%d_parent.bin", S);
            snprintf(name2, sizeof name2, "stats%d_sizes.bin", S);
            if ((rc = dump_state(j, name, name2))) return rc;
        }
        if ((rc = mate_union_and_plan(j->d_parent, N, j->d_size, j->bounds, j->arena, j->st, &j->pe_rounds))) return rc;
    }
    if (j->checks) {  // every read's parent a root (or BAD) after the final compression
        unsigned long long *dc = j->arena.alloc<unsigned long long>(1);
        uint64_t bad = 0;
        if (!dc) return set_error(MP_ENOMEM, "device memory");
        if ((rc = count_nonroot(j->d_parent, N, dc, j->st, &bad))) return rc;
        if (bad) return set_error(MP_EDEVICE, "check: %llu reads' parents are not roots after the mate union",
                                  (unsigned long long)bad);
    }
    j->arena.release_scratch();
    snprintf(name, sizeof name, "stats%d_parent.bin", S + 1);
    snprintf(name2, sizeof name2, "stats%d_sizes.bin", S + 1);
    if ((rc = dump_state(j, name, name2))) return rc;
    j->partitioned = true;
    if (bounds_out) memcpy(bounds_out, j->bounds, sizeof j->bounds);
    return 0;
}

int mp_job_labels(mp_job *j, uint32_t *out)
{
    if (!j || !out || !j->partitioned) return set_error(MP_EARG, "no partition result in this job");
    MP_CUDA(cudaMemcpyAsync(out, j->d_parent, j->pr.n_reads * 4, cudaMemcpyDeviceToHost, j->st));
    MP_CUDA(cudaStreamSynchronize(j->st));
    return 0;
}

namespace {

// The partition files' layout (once per partition).
int plan_job_output(mp_job *j)
{
    if (j->output_ready) return 0;
    StageTimer tm(j->st, j->stage_ms, 7);
    j->stage_ms[7] = 0;
    int rc = plan_output(j->d_fq, j->pr, j->d_parent, j->bounds, j->chunk_rec.data(), j->nchunks, j->T, j->interleaved,
                         &j->out_plan, j->out_sizes, j->arena, j->st);
    j->arena.release_scratch();
    if (rc) return rc;
    j->out_total = j->out_plan.total;
    j->output_ready = true;
    return 0;
}

// The partition files in HBM (once per partition).
int materialize_output(mp_job *j)
{
    if (j->d_out) return 0;
    StageTimer tm(j->st, j->stage_ms, 7);
    j->d_out = j->arena.alloc_persistent<uint8_t>(j->out_total + 16);
    if (!j->d_out) return set_error(MP_ENOMEM, "device memory for the output bytes");
    return copy_output(j->out_plan, j->d_fq, j->d_out, j->st);
}

// The files built in HBM in batches of entries; each batch's bytes go down on the copy stream while the
// next batch is built (copying records straight into mapped host memory from the kernel was slower: the
// small writes use the host link worse than the copy engine).
int materialize_and_download(mp_job *j, uint8_t *out)
{
    constexpr int K = 8;
    const OutputPlan &pl = j->out_plan;
    if (pl.n < (uint64_t)K * 1024 || pl.total == 0) {
        int rc = materialize_output(j);
        if (rc) return rc;
        MP_CUDA(cudaMemcpyAsync(out, j->d_out, j->out_total, cudaMemcpyDeviceToHost, j->st));
        MP_CUDA(cudaStreamSynchronize(j->st));
        return 0;
    }
    if (!j->copy_st && cudaStreamCreateWithFlags(&j->copy_st, cudaStreamNonBlocking) != cudaSuccess) {
        j->copy_st = nullptr;
        return set_error(MP_ECUDA, "cannot create a stream");
    }
    uint64_t e[K + 1], o[K + 1];
    for (int b = 0; b <= K; b++) e[b] = pl.n * (uint64_t)b / K;
    for (int b = 0; b < K; b++) MP_CUDA(cudaMemcpyAsync(&o[b], pl.off + e[b], 8, cudaMemcpyDeviceToHost, j->st));
    o[K] = pl.total;
    j->d_out = j->arena.alloc_persistent<uint8_t>(pl.total + 16);
    if (!j->d_out) return set_error(MP_ENOMEM, "device memory for the output bytes");
    MP_CUDA(cudaStreamSynchronize(j->st));
    cudaEvent_t ev[K];
    for (auto &x : ev) cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
    int rc = 0;
    {
        StageTimer tm(j->st, j->stage_ms, 7);
        for (int b = 0; b < K && !rc; b++) {
            rc = copy_output_range(pl, e[b], e[b + 1], j->d_fq, j->d_out, j->st);
            cudaEventRecord(ev[b], j->st);
            cudaStreamWaitEvent(j->copy_st, ev[b], 0);
            if (!rc && cudaMemcpyAsync(out + o[b], j->d_out + o[b], o[b + 1] - o[b], cudaMemcpyDeviceToHost, j->copy_st) !=
                           cudaSuccess)
                rc = set_error(MP_ECUDA, "copy of the partition files");
        }
    }
    cudaStreamSynchronize(j->copy_st);
    cudaStreamSynchronize(j->st);
    for (auto &x : ev) cudaEventDestroy(x);
    MP_CUDA(cudaGetLastError());
    return rc;
}

}  // namespace

int mp_job_output(mp_job *j, char *out, uint64_t capacity, uint64_t *file_sizes, uint64_t *total)
{
    if (!j || !j->partitioned) return set_error(MP_EARG, "no partition result in this job");
    MP_CUDA(cudaSetDevice(j->ctx->device));
    int rc = plan_job_output(j);
    if (rc) return rc;
    if (file_sizes) memcpy(file_sizes, j->out_sizes.data(), j->out_sizes.size() * 8);
    if (total) *total = j->out_total;
    if (out) {
        if (capacity < j->out_total) return set_error(MP_EARG, "output buffer too small");
        if (j->d_out) {
            MP_CUDA(cudaMemcpyAsync(out, j->d_out, j->out_total, cudaMemcpyDeviceToHost, j->st));
            MP_CUDA(cudaStreamSynchronize(j->st));
        } else if ((rc = materialize_and_download(j, (uint8_t *)out))) {
            return rc;
        }
    }
    return 0;
}

int mp_job_output_device(mp_job *j, const void **d_out, uint64_t *file_sizes, uint64_t *total)
{
    if (!j || !j->partitioned) return set_error(MP_EARG, "no partition result in this job");
    MP_CUDA(cudaSetDevice(j->ctx->device));
    int rc = plan_job_output(j);
    if (!rc) rc = materialize_output(j);
    if (rc) return rc;
    MP_CUDA(cudaStreamSynchronize(j->st));
    if (d_out) *d_out = j->d_out;
    if (file_sizes) memcpy(file_sizes, j->out_sizes.data(), j->out_sizes.size() * 8);
    if (total) *total = j->out_total;
    return 0;
}

int mp_job_kmer_cache_pieces(const mp_job *j) { return j ? (int)j->kc.size() : 0; }

int mp_job_set_kmer_cache(mp_job *j, int enable)
{
    if (!j) return set_error(MP_EARG, "null job");
    j->store = enable ? STORE_KMER_CACHE : STORE_FASTQ;
    if (!enable) drop_kmer_cache(j);
    return 0;
}

int mp_job_set_read_store(mp_job *j, int store)
{
    if (!j) return set_error(MP_EARG, "null job");
    if (store != MP_STORE_FASTQ && store != MP_STORE_KMER_CACHE && store != MP_STORE_PACKED)
        return set_error(MP_EARG, "unknown read store %d", store);
    if (store != j->store) drop_kmer_cache(j);
    j->store = store;
    return 0;
}

int mp_job_read_store(const mp_job *j)
{
    if (!j) return set_error(MP_EARG, "null job");
    if (j->kc.empty()) return MP_STORE_FASTQ;
    return j->kc[0].pw ? MP_STORE_PACKED : MP_STORE_KMER_CACHE;
}

int mp_job_set_wait_limits(mp_job *j, uint32_t lookback_spins, uint32_t union_retries, uint32_t mate_rounds)
{
    if (!j) return set_error(MP_EARG, "null job");
    const WaitLimits d;
    j->arena.lim.lookback_spins = lookback_spins ? lookback_spins : d.lookback_spins;
    j->arena.lim.union_retries = union_retries ? union_retries : d.union_retries;
    j->arena.lim.mate_rounds = mate_rounds ? mate_rounds : d.mate_rounds;
    return 0;
}

int mp_job_set_checks(mp_job *j, int on)
{
    if (!j) return set_error(MP_EARG, "null job");
    j->checks = on != 0;
    return 0;
}

int mp_count_unsorted(mp_ctx *ctx, const uint64_t *lo, const uint8_t *hi, uint64_t n, void *stream, uint64_t *out)
{
    if (!ctx || !out || (n && !lo)) return set_error(MP_EARG, "null argument");
    MP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    DeviceArena arena;
    arena.st = st;
    arena.budget_used = &ctx->used;
    arena.budget_limit = ctx->budget;
    unsigned long long *dc = arena.alloc<unsigned long long>(1);
    if (!dc) return set_error(MP_ENOMEM, "device memory");
    const int rc = count_unsorted(lo, hi, n, dc, st, out);
    arena.release_all();
    return rc;
}

int mp_job_set_scan_piece_tuples(mp_job *j, uint64_t max_tuples)
{
    if (!j) return set_error(MP_EARG, "null job");
    j->piece_tuples = max_tuples;
    return 0;
}

int mp_job_scan_pieces(const mp_job *j) { return j ? j->pieces_total : 0; }

int mp_job_set_dump_dir(mp_job *j, const char *dir)
{
    if (!j) return set_error(MP_EARG, "null job");
    j->dump_dir = dir ? dir : "";
    return 0;
}

int mp_job_stage_ms(const mp_job *j, double *ms, int n)
{
    if (!j || !ms) return set_error(MP_EARG, "null argument");
    for (int i = 0; i < n && i < 8; i++) ms[i] = j->stage_ms[i];
    return 0;
}

int mp_job_sort_stats(const mp_job *j, uint64_t *tuples, int *passes, double *pass_ms, uint64_t *bytes)
{
    if (!j) return set_error(MP_EARG, "null job");
    if (tuples) *tuples = j->sort_tuples_total;
    if (passes) *passes = j->sort_passes_total;
    if (pass_ms) *pass_ms = j->sort_ms_total;
    if (bytes) *bytes = j->sort_bytes_total;
    return 0;
}

int mp_job_sort_split(const mp_job *j, double *pass_ms, double *unit_ms, double *big_ms, uint64_t *units,
                      uint64_t *big_buckets, uint64_t *big_tuples, uint64_t *unit_counters)
{
    if (!j) return set_error(MP_EARG, "null job");
    if (unit_counters) {
        unit_counters[0] = j->unit_passes_total;
        for (int q = 0; q < 3; q++) unit_counters[1 + q] = j->phase_total[q];
        for (int q = 0; q < 7; q++) unit_counters[4 + q] = j->pass_cycles_total[q];
    }
    if (pass_ms) *pass_ms = j->sort_ms_total;
    if (unit_ms) *unit_ms = j->seg_ms_total;
    if (big_ms) *big_ms = j->big_ms_total;
    if (units) *units = j->units_total;
    if (big_buckets) *big_buckets = j->big_buckets_total;
    if (big_tuples) *big_tuples = j->big_tuples_total;
    return 0;
}

int mp_sort_tuples(mp_ctx *ctx, const uint64_t *lo_in, const uint8_t *hi_in, const uint32_t *id_in, uint64_t *lo_out,
                   uint8_t *hi_out, uint32_t *id_out, uint64_t n, void *stream)
{
    if (!ctx || !lo_in || !id_in || !lo_out || !id_out) return set_error(MP_EARG, "null argument");
    if ((hi_in == nullptr) != (hi_out == nullptr)) return set_error(MP_EARG, "hi_in and hi_out must both be given or both NULL");
    MP_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t st = (cudaStream_t)stream;
    DeviceArena arena;
    arena.st = st;
    arena.budget_used = &ctx->used;
    arena.budget_limit = ctx->budget;
    const bool has_hi = hi_in != nullptr;
    SortBufs b;
    b.lo[0] = lo_out;
    b.id[0] = id_out;
    b.hi[0] = hi_out;
    b.lo[1] = arena.alloc<uint64_t>(n + 1);
    b.id[1] = arena.alloc<uint32_t>(n + 1);
    b.hi[1] = has_hi ? arena.alloc<uint8_t>(n + 1) : nullptr;
    if (!b.lo[1] || !b.id[1] || (has_hi && !b.hi[1])) {
        arena.release_all();
        return set_error(MP_ENOMEM, "device memory for sorting %llu tuples", (unsigned long long)n);
    }
    if (n) {
        MP_CUDA(cudaMemcpyAsync(lo_out, lo_in, n * 8, cudaMemcpyDeviceToDevice, st));
        MP_CUDA(cudaMemcpyAsync(id_out, id_in, n * 4, cudaMemcpyDeviceToDevice, st));
        if (has_hi) MP_CUDA(cudaMemcpyAsync(hi_out, hi_in, n, cudaMemcpyDeviceToDevice, st));
    }
    int rc = radix_sort(b, n, has_hi, arena, st, nullptr);
    if (!rc && b.cur == 1 && n) {
        cudaMemcpyAsync(lo_out, b.lo[1], n * 8, cudaMemcpyDeviceToDevice, st);
        cudaMemcpyAsync(id_out, b.id[1], n * 4, cudaMemcpyDeviceToDevice, st);
        if (has_hi) cudaMemcpyAsync(hi_out, b.hi[1], n, cudaMemcpyDeviceToDevice, st);
    }
    arena.release_all();
    cudaError_t e = cudaStreamSynchronize(st);
    if (!rc && e != cudaSuccess) rc = set_cuda_error(e, "mp_sort_tuples", __FILE__, __LINE__);
    return rc;
}

// ------------------------------------------------------------- chunk index

// genFastqIdx (genFastqIdx.c:142-376) for single-end / interleaved files held in memory.
int mp_fastq_index(int num_chunks, int n_pe, int n_se, int n_il, int nfiles, const char *const *files,
                   const uint64_t *sizes, int32_t *out_file_no, uint64_t *out_offsets, int *out_count)
{
    if (!files || !sizes || !out_file_no || !out_offsets || !out_count || nfiles < 1 || num_chunks < 1)
        return set_error(MP_EARG, "bad argument");
    if (n_pe != 0) return set_error(MP_EUNSUP, "two-file paired-end input is not supported");
    if (n_se + n_il != nfiles || n_se < 0 || n_il < 0) return set_error(MP_EARG, "file counts do not match the file list");
    if (n_se && n_il) return set_error(MP_EUNSUP, "mixing single-end and interleaved files is not supported");
    uint64_t total = 0;
    for (int i = 0; i < nfiles; i++) total += sizes[i];
    const uint64_t per = total / (uint64_t)num_chunks;
    int max_read = 300, interleaved = 0, nrec = 0;
    int32_t fno = 0;
    uint64_t ofs = 0;
    for (int c = 0; c < num_chunks; c++) {
        uint64_t rem = per * (uint64_t)c;  // getFileIndex (:28-53)
        fno = 0;
        while (rem >= sizes[fno]) { rem -= sizes[fno]; fno++; }
        ofs = rem;
        if (fno >= n_se) interleaved = 1;
        if (sizes[fno] - ofs < (uint64_t)max_read) {
            if (fno + 1 == nfiles) break;
            fno++;
            ofs = 0;
        }
        if (c == 0) {
            out_file_no[nrec] = fno;
            out_offsets[nrec++] = ofs;
            continue;
        }
        // record boundary search in a 3000-byte read of the file (:254-307); bytes past the
        // read count as zero, as in a zero-filled buffer
        const char *base = files[fno] + ofs;
        const uint64_t avail = sizes[fno] - ofs, nread = avail < 3000 ? avail : 3000;
        if (nread <= (uint64_t)max_read) return set_error(MP_EFMT, "chunk %d starts too close to a file end", c);
        const uint64_t CAP = 5000;
        auto at = [&](uint64_t i) -> int { return i < nread ? (unsigned char)base[i] : 0; };
        uint64_t jj = 0;
        int flag = 0, kk = 0, found = 0;
        for (jj = 0; jj < nread; jj++) {
            if (at(jj) == '\n' && at(jj + 1) == '+') {
                flag = 1;
                jj += 2;
                while (jj < CAP && at(jj) != '\n') jj++;
                jj++;
            }
            kk = 0;
            if (flag && at(jj) == '\n') {
                jj++;
                kk++;
                if (interleaved) {
                    uint64_t q = jj;
                    std::string a, b;
                    while (q < CAP && at(q) != '/' && at(q) != ' ') a.push_back((char)at(q++));
                    for (int l = 0; l < 4; l++) {
                        while (q < CAP && at(q) != '\n') q++;
                        q++;
                    }
                    const uint64_t j2 = q;
                    while (q < CAP && at(q) != ' ' && at(q) != '/') b.push_back((char)at(q++));
                    if (q >= CAP) return set_error(MP_EFMT, "mate names not found near chunk %d", c);
                    kk = (int)q;
                    if (a != b) jj = j2;
                }
                found = 1;
                break;
            }
        }
        if (!found) return set_error(MP_EFMT, "no record boundary within 3000 bytes of chunk %d", c);
        if (2 * kk + 30 < max_read) max_read = 2 * kk + 30;
        out_file_no[nrec] = fno;
        out_offsets[nrec++] = ofs + jj;
    }
    out_file_no[nrec] = nfiles - 1;
    out_offsets[nrec++] = sizes[nfiles - 1];
    *out_count = nrec;
    return 0;
}

}  // extern "C"
