// Request loop over one context: continuous admission of partition jobs by HBM footprint.
//
// Each worker thread owns one mp_job (and so one CUDA stream).  A request is admitted when a
// worker is free and its estimated device footprint fits in what the budget has left; admitted
// jobs run the whole stage chain -- chunk index, upload, m-mer histogram, partition, partition
// FASTQ download -- on their own streams, so the kernels of different jobs overlap on the GPU.
// The reference runs one input per MPI launch and has no counterpart of this loop.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "metapart_gpu.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket = 0;
    const char *fastq = nullptr;
    uint64_t nbytes = 0;
    mp_request_params p{};
    char *out = nullptr;
    uint64_t out_cap = 0;
    uint64_t *file_sizes = nullptr;
    uint32_t *labels = nullptr;
    uint64_t labels_cap = 0;
    uint64_t footprint = 0;
    bool exclusive = false;  // retried alone after running out of budget beside other jobs
    double t_submit = 0;
};

double ms_since(Clock::time_point t0) { return std::chrono::duration<double, std::milli>(Clock::now() - t0).count(); }

// Bytes per record and bases per record of the first records (at most 256 or 1 MB).
void sample_records(const char *b, uint64_t n, double *rec_bytes, double *bases)
{
    uint64_t i = 0, recs = 0, seq = 0;
    const uint64_t lim = n < (1u << 20) ? n : (1u << 20);
    while (i < lim && recs < 256) {
        uint64_t line[4], st = i;
        int l = 0;
        for (; l < 4 && i < lim; l++) {
            const char *e = (const char *)memchr(b + i, '\n', lim - i);
            if (!e) break;
            line[l] = (uint64_t)(e - (b + i));
            i = (uint64_t)(e - b) + 1;
        }
        if (l < 4) {
            i = st;
            break;
        }
        seq += line[1];
        recs++;
    }
    if (recs == 0) {
        *rec_bytes = 8;
        *bases = 1;
        return;
    }
    *rec_bytes = (double)i / (double)recs;
    *bases = (double)seq / (double)recs;
}

}  // namespace

struct mp_server {
    mp_ctx *ctx = nullptr;
    uint64_t budget = 0;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request> queue;
    std::unordered_map<uint64_t, mp_result> done;
    std::unordered_set<uint64_t> open;  // tickets issued whose results have not been released yet
    std::vector<std::thread> workers;
    uint64_t next_ticket = 1;
    uint64_t reserved = 0, peak_reserved = 0;
    uint64_t admitted = 0, completed = 0;
    int running = 0, peak_running = 0;
    bool stop = false;
};

namespace {

void run_request(mp_server *s, mp_job *job, Request &rq, mp_result &res)
{
    const mp_request_params &p = rq.p;
    const int C = p.num_chunks;
    std::vector<int32_t> fno(C + 1);
    std::vector<uint64_t> ofs(C + 1), starts, first(C + 1), bounds(17);
    static thread_local std::vector<uint64_t> hist;
    hist.resize(MP_NUM_BUCKETS + 1);
    int nrec = 0;
    const char *files[1] = {rq.fastq};
    int rc = mp_fastq_index(C, 0, p.interleaved ? 0 : 1, p.interleaved ? 1 : 0, 1, files, &rq.nbytes, fno.data(),
                            ofs.data(), &nrec);
    if (!rc && nrec != C + 1) rc = MP_EFMT;
    if (!rc) rc = mp_job_set_read_store(job, p.read_store);
    if (!rc) {
        starts.assign(ofs.begin(), ofs.begin() + nrec);
        starts[nrec - 1] = rq.nbytes;
        std::vector<uint64_t> reads(C);
        rc = mp_job_load_count(job, rq.fastq, rq.nbytes, &rq.nbytes, 1, p.interleaved, p.k, p.min3, starts.data(), C,
                               hist.data(), reads.data());
        first[0] = 0;
        for (int c = 0; c < C && !rc; c++) first[c + 1] = first[c] + reads[c];
    }
    if (!rc) {
        mp_part_params pp = {p.k, p.min3, p.num_scans, p.num_threads};
        rc = mp_job_partition(job, &pp, starts.data(), first.data(), C, hist.data(), bounds.data());
    }
    res.n_reads = mp_job_num_reads(job);
    if (!rc && rq.labels) {
        if (rq.labels_cap < res.n_reads) rc = MP_EARG;
        else rc = mp_job_labels(job, rq.labels);
    }
    if (!rc) rc = mp_job_output(job, rq.out, rq.out_cap, rq.file_sizes, &res.out_total);
    if (!rc) {
        memcpy(res.bounds, bounds.data(), sizeof res.bounds);
        double ms[8] = {0};
        mp_job_stage_ms(job, ms, 8);
        for (double v : ms) res.device_ms += v;
    }
    res.status = rc;
    if (rc) snprintf(res.error, sizeof res.error, "%s", mp_last_error());
    mp_job_reset(job);
    (void)s;
}

void worker_main(mp_server *s)
{
    mp_job *job = nullptr;
    const int jrc = mp_job_create(s->ctx, &job);
    for (;;) {
        Request rq;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            for (;;) {
                if (s->stop && s->queue.empty()) {
                    lk.unlock();
                    if (job) mp_job_destroy(job);
                    return;
                }
                if (!s->queue.empty()) {
                    const Request &h = s->queue.front();
                    const bool fits = h.exclusive ? s->running == 0 : s->reserved + h.footprint <= s->budget;
                    if (fits || s->running == 0) break;  // strict FIFO: the head waits for memory
                }
                s->cv_work.wait(lk);
            }
            rq = s->queue.front();
            s->queue.pop_front();
            s->reserved += rq.footprint;
            s->peak_reserved = std::max(s->peak_reserved, s->reserved);
            s->running++;
            s->peak_running = std::max(s->peak_running, s->running);
            s->admitted++;
        }
        mp_result res{};
        res.t_submit_ms = rq.t_submit;
        res.t_admit_ms = ms_since(s->t0);
        res.footprint = rq.footprint;
        if (jrc) {
            res.status = jrc;
            snprintf(res.error, sizeof res.error, "no job: %s", mp_last_error());
        } else {
            run_request(s, job, rq, res);
        }
        res.t_done_ms = ms_since(s->t0);
        std::lock_guard<std::mutex> lk(s->mu);
        s->reserved -= rq.footprint;
        s->running--;
        const bool others = s->running > 0;
        if (res.status == MP_ENOMEM && others && !rq.exclusive) {
            rq.exclusive = true;  // ran out of budget beside other jobs: run again alone
            s->queue.push_front(rq);
            s->admitted--;
        } else {
            s->done[rq.ticket] = res;
            s->completed++;
            s->cv_done.notify_all();
        }
        s->cv_work.notify_all();
    }
}

}  // namespace

extern "C" {

uint64_t mp_request_footprint(const char *fastq, uint64_t nbytes, const mp_request_params *p)
{
    if (!fastq || !p || p->num_scans < 1) return 0;
    double rec_bytes = 0, bases_per = 0;
    sample_records(fastq, nbytes, &rec_bytes, &bases_per);
    const double reads = (double)nbytes / rec_bytes * 1.05 + 64.0;
    const double bases = reads * bases_per;
    const double tuples = bases / p->num_scans * 1.15 + (double)(1 << 20);
    double f = (double)nbytes + 64;                     // FASTQ bytes
    f += reads * (4 * 8 + 20);                          // newline positions (parse scratch) + record table
    f += reads * (9 + 12);                              // parent, size, BAD flags; per-scan k-mer counts and offsets
    f += tuples * 27.0;                                 // two tuple buffers of 13 B + look-back status
    f += (double)nbytes * (p->interleaved ? 2 : 1);     // partition FASTQ
    f += reads * 40.0;                                  // output entries and their sort
    if (p->read_store == MP_STORE_KMER_CACHE) f += bases * 9.0;            // k-mer cache of the count pass
    else if (p->read_store == MP_STORE_PACKED) f += bases * 0.375 + reads * 8;  // packed reads and their offsets
    f += 64.0 * (1 << 20);                              // histograms, scan scratch
    return (uint64_t)(f * 1.10);
}

int mp_server_create(mp_ctx *ctx, int slots, uint64_t hbm_budget, mp_server **out)
{
    if (!ctx || !out || slots < 1 || slots > 64) return MP_EARG;
    mp_server *s = new mp_server;
    s->ctx = ctx;
    s->budget = hbm_budget ? hbm_budget : ~0ull;
    s->t0 = Clock::now();
    for (int i = 0; i < slots; i++) s->workers.emplace_back(worker_main, s);
    *out = s;
    return 0;
}

int mp_server_submit(mp_server *s, const char *fastq, uint64_t nbytes, const mp_request_params *p, char *out,
                     uint64_t out_cap, uint64_t *file_sizes, uint32_t *labels, uint64_t labels_cap, uint64_t *ticket)
{
    if (!s || !fastq || !p || !ticket || p->num_chunks < 1 || p->num_threads < 1) return MP_EARG;
    Request rq;
    rq.fastq = fastq;
    rq.nbytes = nbytes;
    rq.p = *p;
    rq.out = out;
    rq.out_cap = out_cap;
    rq.file_sizes = file_sizes;
    rq.labels = labels;
    rq.labels_cap = labels_cap;
    rq.footprint = mp_request_footprint(fastq, nbytes, p);
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return MP_EARG;
    if (rq.footprint > s->budget) rq.exclusive = true;  // larger than the budget: alone, and the job's own checks decide
    rq.ticket = s->next_ticket++;
    rq.t_submit = ms_since(s->t0);
    s->open.insert(rq.ticket);
    s->queue.push_back(rq);
    *ticket = rq.ticket;
    s->cv_work.notify_all();
    return 0;
}

int mp_server_poll(mp_server *s, uint64_t ticket, int wait, mp_result *res)
{
    if (!s || !res) return MP_EARG;
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        auto it = s->done.find(ticket);
        if (it != s->done.end()) {
            *res = it->second;
            s->done.erase(it);
            s->open.erase(ticket);
            s->cv_done.notify_all();  // other waiters on this ticket see it released
            return 1;
        }
        if (!s->open.count(ticket)) return MP_EARG;  // never issued, or its result was released already
        if (!wait) return 0;
        s->cv_done.wait(lk);
    }
}

int mp_server_stats(mp_server *s, mp_server_stats_t *st)
{
    if (!s || !st) return MP_EARG;
    std::lock_guard<std::mutex> lk(s->mu);
    st->queued = s->queue.size();
    st->running = s->running;
    st->peak_running = s->peak_running;
    st->admitted = s->admitted;
    st->completed = s->completed;
    st->reserved = s->reserved;
    st->peak_reserved = s->peak_reserved;
    st->budget = s->budget;
    return 0;
}

void mp_server_destroy(mp_server *s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
    }
    for (auto &t : s->workers) t.join();
    delete s;
}

}  // extern "C"
