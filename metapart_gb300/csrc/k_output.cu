// K7: partition FASTQ output (writeOutput3, metapart.c:956-1066).
//
// Output file j = partition * T + tid holds, in input order, every record whose
// component root falls in the partition's read-id range, written by thread tid (the
// thread owning the record's chunk).  An interleaved pair is written to the partition of
// mate 1's root and, when mate 2's root differs, again to mate 2's (:1006-1047).  On the
// GPU each (file, unit) entry is generated in input order, entries are stably sorted by
// file, their byte offsets come from one exclusive scan, and a warp copies each record.
#include "k_output.cuh"
#include "k_sort.cuh"

namespace mp {

__device__ __forceinline__ uint32_t part_of(const uint64_t *bounds, uint32_t root)
{
    uint32_t p = 0;
    while (p < 16 && !((uint64_t)root < bounds[p + 1])) p++;
    return p;
}

struct OutCtx {
    const uint64_t *rec_start;
    const uint32_t *label;
    const uint64_t *bounds;    // 17
    const uint64_t *chunk_rec; // nchunks + 1
    int nchunks, T, per_thread, interleaved;
    uint64_t units;
};

__device__ __forceinline__ uint32_t tid_of(const OutCtx &c, uint64_t rec)
{
    int lo = 0, hi = c.nchunks - 1;
    while (lo < hi) {
        int m = (lo + hi + 1) >> 1;
        if (c.chunk_rec[m] <= rec) lo = m; else hi = m - 1;
    }
    return (uint32_t)(lo / c.per_thread);
}

// entries per unit (1 or 2) and the file of each
__global__ void k_out_dest(OutCtx c, uint32_t *nent, uint32_t *f1, uint32_t *f2)
{
    const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= c.units) return;
    const uint64_t r = c.interleaved ? 2 * u : u;
    const uint32_t t = tid_of(c, r);
    const uint32_t pu = c.label[r];
    f1[u] = part_of(c.bounds, pu) * c.T + t;
    uint32_t ne = 1;
    if (c.interleaved) {
        const uint32_t pv = c.label[r + 1];
        if (pu != pv) {
            f2[u] = part_of(c.bounds, pv) * c.T + t;
            ne = 2;
        }
    }
    nent[u] = ne;
}

__global__ void k_out_entries(OutCtx c, const uint32_t *f1, const uint32_t *f2, const uint32_t *nent,
                              const uint64_t *eoff, uint64_t *key, uint32_t *val)
{
    const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= c.units) return;
    const uint64_t o = eoff[u];
    key[o] = f1[u];
    val[o] = (uint32_t)u;
    if (nent[u] == 2) {
        key[o + 1] = f2[u];
        val[o + 1] = (uint32_t)u;
    }
}

// Entry lengths; file sizes by one atomic per file and warp (entries are sorted by file, so a
// warp's lanes of one file are contiguous: the last lane adds its segment of an inclusive scan).
__global__ void k_out_len(OutCtx c, const uint32_t *val, uint64_t n, uint64_t *len, const uint64_t *key,
                          unsigned long long *file_bytes)
{
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool v = i < n;
    uint64_t l = 0, f = ~0ull;
    if (v) {
        const uint64_t u = val[i];
        const uint64_t r0 = c.interleaved ? 2 * u : u, r1 = c.interleaved ? 2 * u + 2 : u + 1;
        l = c.rec_start[r1] - c.rec_start[r0];
        len[i] = l;
        f = key[i];
    }
    uint64_t incl = l;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += y;
    }
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, f);
    const int first = __ffs(peers) - 1, last = 31 - __clz(peers);
    const uint64_t before = __shfl_sync(0xFFFFFFFFu, incl, first > 0 ? first - 1 : 0);
    if (v && lane == last) atomicAdd(&file_bytes[f], (unsigned long long)(incl - (first > 0 ? before : 0)));
}

// One record (l bytes at fq + s) to out + o by a warp.
__device__ __forceinline__ void copy_record(const uint8_t *fq, uint64_t s, uint64_t l, uint64_t o, uint8_t *out, int lane)
{
    const uint64_t head = min(l, (uint64_t)((4 - (o & 3)) & 3));
    if ((uint64_t)lane < head) out[o + lane] = fq[s + lane];
    const uint64_t words = (l - head) >> 2;
    const uint64_t sb = s + head;
    const uint32_t a = (uint32_t)(sb & 3) * 8;
    const uint32_t *src = reinterpret_cast<const uint32_t *>(fq + (sb & ~3ull));
    uint32_t *dst = reinterpret_cast<uint32_t *>(out + o + head);
    for (uint64_t j = lane; j < words; j += 32) dst[j] = __funnelshift_r(src[j], src[j + 1], a);
    const uint64_t t0 = head + (words << 2);
    if ((uint64_t)lane < l - t0) out[o + t0 + lane] = fq[s + t0 + lane];
}

constexpr int OC_PER_WARP = 8;  // records per warp in k_out_copy

// A warp copies OC_PER_WARP records: lanes fetch the records' source ranges and destinations in one
// round, then for each record: bytes up to the first 4-byte boundary of the destination, aligned
// 4-byte words assembled from two aligned source words by a funnel shift, the tail bytes.  Source
// words may reach 3 bytes past the record; the FASTQ buffer carries 64 bytes of padding.
__global__ void k_out_copy(OutCtx c, const uint8_t *fq, const uint32_t *val, const uint64_t *off, uint64_t n, uint8_t *out)
{
    const uint64_t w0 = (((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * OC_PER_WARP;
    const int lane = threadIdx.x & 31;
    if (w0 >= n) return;
    uint64_t my_s = 0, my_l = 0, my_o = 0;  // lane q < OC_PER_WARP: record w0 + q
    if (lane < OC_PER_WARP && w0 + lane < n) {
        const uint64_t u = val[w0 + lane];
        const uint64_t r0 = c.interleaved ? 2 * u : u, r1 = c.interleaved ? 2 * u + 2 : u + 1;
        my_s = c.rec_start[r0];
        my_l = c.rec_start[r1] - my_s;
        my_o = off[w0 + lane];
    }
    const int nrec = (int)min((uint64_t)OC_PER_WARP, n - w0);
    for (int q = 0; q < nrec; q++) {
        const uint64_t s = __shfl_sync(0xFFFFFFFFu, my_s, q), l = __shfl_sync(0xFFFFFFFFu, my_l, q),
                       o = __shfl_sync(0xFFFFFFFFu, my_o, q);
        copy_record(fq, s, l, o, out, lane);
    }
}

int plan_output(const uint8_t *d_fq, const ParsedReads &pr, const uint32_t *d_label, const uint64_t *bounds_host,
                const uint64_t *chunk_rec_host, int nchunks, int T, int interleaved, OutputPlan *plan,
                std::vector<uint64_t> &file_sizes, DeviceArena &arena, cudaStream_t st)
{
    (void)d_fq;
    const uint64_t units = interleaved ? pr.n_reads / 2 : pr.n_reads;
    const int nf = 16 * T;
    file_sizes.assign(nf, 0);
    OutCtx c;
    c.rec_start = pr.rec_start;
    c.label = d_label;
    c.nchunks = nchunks;
    c.T = T;
    c.per_thread = nchunks / T;
    c.interleaved = interleaved;
    c.units = units;
    uint64_t *bounds = arena.alloc<uint64_t>(17), *chunk_rec = arena.alloc<uint64_t>(nchunks + 1);
    uint32_t *nent = arena.alloc<uint32_t>(units + 1), *f1 = arena.alloc<uint32_t>(units + 1),
             *f2 = arena.alloc<uint32_t>(units + 1);
    uint64_t *eoff = arena.alloc<uint64_t>(units + 1), *ntot = arena.alloc<uint64_t>(1);
    unsigned long long *fbytes = arena.alloc<unsigned long long>(nf);
    size_t tb = scan_tmp_bytes(2 * units + 2);
    void *tmp = arena.alloc<uint8_t>(tb);
    if (!bounds || !chunk_rec || !nent || !f1 || !f2 || !eoff || !ntot || !fbytes || !tmp)
        return set_error(MP_ENOMEM, "device memory for the output gather");
    MP_CUDA(cudaMemcpyAsync(bounds, bounds_host, 17 * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    MP_CUDA(cudaMemcpyAsync(chunk_rec, chunk_rec_host, (nchunks + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, st));
    MP_CUDA(cudaMemsetAsync(fbytes, 0, nf * sizeof(unsigned long long), st));
    c.bounds = bounds;
    c.chunk_rec = chunk_rec;
    const unsigned gb = (unsigned)((units + 255) / 256);
    (mp::count_launch(), k_out_dest<<<gb, 256, 0, st>>>(c, nent, f1, f2));
    scan_u32_to_u64(nent, eoff, units, ntot, tmp, tb, st);
    uint64_t n = 0;
    MP_CUDA(cudaMemcpyAsync(&n, ntot, sizeof n, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    SortBufs sb;
    for (int i = 0; i < 2; i++) {
        sb.lo[i] = arena.alloc<uint64_t>(n + 1);
        sb.id[i] = arena.alloc<uint32_t>(n + 1);
        if (!sb.lo[i] || !sb.id[i]) return set_error(MP_ENOMEM, "device memory for the output entries");
    }
    (mp::count_launch(), k_out_entries<<<gb, 256, 0, st>>>(c, f1, f2, nent, eoff, sb.lo[0], sb.id[0]));
    int rc = radix_sort(sb, n, false, arena, st, nullptr);
    if (rc) return rc;
    uint64_t *len = arena.alloc<uint64_t>(n + 1);
    plan->val = arena.alloc_persistent<uint32_t>(n + 1);
    plan->off = arena.alloc_persistent<uint64_t>(n + 1);
    size_t tb2 = scan_tmp_bytes(n + 1);
    void *tmp2 = arena.alloc<uint8_t>(tb2);
    if (!len || !plan->val || !plan->off || !tmp2) return set_error(MP_ENOMEM, "device memory for the output offsets");
    const unsigned ge = (unsigned)((n + 255) / 256);
    (mp::count_launch(), k_out_len<<<ge, 256, 0, st>>>(c, sb.id[sb.cur], n, len, sb.lo[sb.cur], fbytes));
    scan_u64(len, plan->off, n, ntot, tmp2, tb2, st);
    MP_CUDA(cudaMemcpyAsync(plan->val, sb.id[sb.cur], n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    uint64_t total = 0;
    MP_CUDA(cudaMemcpyAsync(&total, ntot, sizeof total, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaMemcpyAsync(file_sizes.data(), fbytes, nf * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    plan->n = n;
    plan->total = total;
    plan->rec_start = pr.rec_start;
    plan->interleaved = interleaved;
    return 0;
}

// ------------------------------------------------------ batches of samples

// Samples one after another in the read ids; sample q's files are the global files file0[q] + j.
struct BatchOutCtx {
    const uint32_t *label;
    const uint64_t *srec;       // nseg + 1 read offsets
    const uint64_t *bounds;     // nseg x 17, each sample's own read ids
    const uint64_t *chunk_rec;  // every sample's nchunks + 1 chunk record starts (its own read ids), one after another
    const uint32_t *chunk0;     // nseg + 1: where each sample's chunk records start in chunk_rec
    const uint32_t *T, *per_thread, *file0;  // per sample
    int nseg, interleaved;
    uint64_t units;
};

__device__ __forceinline__ uint32_t seg_of(const uint64_t *srec, int nseg, uint64_t r)
{
    int lo = 0, hi = nseg - 1;  // the last sample starting at or below r
    while (lo < hi) {
        const int m = (lo + hi + 1) >> 1;
        if (srec[m] <= r) lo = m; else hi = m - 1;
    }
    return (uint32_t)lo;
}

__global__ void k_outb_dest(BatchOutCtx c, uint32_t *nent, uint32_t *f1, uint32_t *f2)
{
    const uint64_t u = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= c.units) return;
    const uint64_t r = c.interleaved ? 2 * u : u;
    const uint32_t q = seg_of(c.srec, c.nseg, r);
    const uint64_t R = c.srec[q], lr = r - R;
    const uint64_t *cr = c.chunk_rec + c.chunk0[q];
    int lo = 0, hi = (int)(c.chunk0[q + 1] - c.chunk0[q]) - 2;  // the sample's chunk holding lr
    while (lo < hi) {
        const int m = (lo + hi + 1) >> 1;
        if (cr[m] <= lr) lo = m; else hi = m - 1;
    }
    const uint32_t t = (uint32_t)lo / c.per_thread[q], T = c.T[q];
    const uint64_t *b = c.bounds + (uint64_t)q * 17;
    const uint32_t pu = c.label[r];
    f1[u] = c.file0[q] + part_of(b, (uint32_t)(pu - R)) * T + t;
    uint32_t ne = 1;
    if (c.interleaved) {
        const uint32_t pv = c.label[r + 1];
        if (pu != pv) {
            f2[u] = c.file0[q] + part_of(b, (uint32_t)(pv - R)) * T + t;
            ne = 2;
        }
    }
    nent[u] = ne;
}

int plan_output_batch(const ParsedReads &pr, const uint32_t *d_label, int interleaved, const std::vector<uint64_t> &seg_reads,
                      const std::vector<uint64_t> &bounds_host, const std::vector<std::vector<uint64_t>> &chunk_rec_host,
                      const std::vector<int> &T, OutputPlan *plan, std::vector<uint64_t> &file_sizes,
                      std::vector<uint64_t> &file0, DeviceArena &arena, cudaStream_t st)
{
    const int nseg = (int)seg_reads.size() - 1;
    const uint64_t units = interleaved ? pr.n_reads / 2 : pr.n_reads;
    std::vector<uint32_t> c0(nseg + 1, 0), hT(nseg), hpt(nseg), hf0(nseg);
    std::vector<uint64_t> crec;
    file0.assign(nseg + 1, 0);
    for (int q = 0; q < nseg; q++) {
        const int nch = (int)chunk_rec_host[q].size() - 1;
        if (nch < 1 || T[q] < 1 || nch % T[q]) return set_error(MP_EARG, "sample %d: numThreads must divide its chunks", q);
        c0[q] = (uint32_t)crec.size();
        crec.insert(crec.end(), chunk_rec_host[q].begin(), chunk_rec_host[q].end());
        hT[q] = (uint32_t)T[q];
        hpt[q] = (uint32_t)(nch / T[q]);
        hf0[q] = (uint32_t)file0[q];
        file0[q + 1] = file0[q] + 16ull * (uint64_t)T[q];
    }
    c0[nseg] = (uint32_t)crec.size();
    const uint64_t nf = file0[nseg];
    file_sizes.assign(nf, 0);
    uint64_t *srec = arena.alloc<uint64_t>(nseg + 1), *bnd = arena.alloc<uint64_t>((size_t)nseg * 17);
    uint64_t *dcr = arena.alloc<uint64_t>(crec.size());
    uint32_t *dc0 = arena.alloc<uint32_t>(nseg + 1), *dT = arena.alloc<uint32_t>(nseg), *dpt = arena.alloc<uint32_t>(nseg),
             *df0 = arena.alloc<uint32_t>(nseg);
    uint32_t *nent = arena.alloc<uint32_t>(units + 1), *f1 = arena.alloc<uint32_t>(units + 1),
             *f2 = arena.alloc<uint32_t>(units + 1);
    uint64_t *eoff = arena.alloc<uint64_t>(units + 1), *ntot = arena.alloc<uint64_t>(1);
    unsigned long long *fbytes = arena.alloc<unsigned long long>(nf);
    size_t tb = scan_tmp_bytes(2 * units + 2);
    void *tmp = arena.alloc<uint8_t>(tb);
    if (!srec || !bnd || !dcr || !dc0 || !dT || !dpt || !df0 || !nent || !f1 || !f2 || !eoff || !ntot || !fbytes || !tmp)
        return set_error(MP_ENOMEM, "device memory for the output gather");
    MP_CUDA(cudaMemcpyAsync(srec, seg_reads.data(), (nseg + 1) * 8, cudaMemcpyHostToDevice, st));
    MP_CUDA(cudaMemcpyAsync(bnd, bounds_host.data(), (size_t)nseg * 17 * 8, cudaMemcpyHostToDevice, st));
    MP_CUDA(cudaMemcpyAsync(dcr, crec.data(), crec.size() * 8, cudaMemcpyHostToDevice, st));
    MP_CUDA(cudaMemcpyAsync(dc0, c0.data(), (nseg + 1) * 4, cudaMemcpyHostToDevice, st));
    MP_CUDA(cudaMemcpyAsync(dT, hT.data(), nseg * 4, cudaMemcpyHostToDevice, st));
    MP_CUDA(cudaMemcpyAsync(dpt, hpt.data(), nseg * 4, cudaMemcpyHostToDevice, st));
    MP_CUDA(cudaMemcpyAsync(df0, hf0.data(), nseg * 4, cudaMemcpyHostToDevice, st));
    MP_CUDA(cudaMemsetAsync(fbytes, 0, nf * sizeof(unsigned long long), st));
    BatchOutCtx bc;
    bc.label = d_label;
    bc.srec = srec;
    bc.bounds = bnd;
    bc.chunk_rec = dcr;
    bc.chunk0 = dc0;
    bc.T = dT;
    bc.per_thread = dpt;
    bc.file0 = df0;
    bc.nseg = nseg;
    bc.interleaved = interleaved;
    bc.units = units;
    OutCtx c{};
    c.rec_start = pr.rec_start;
    c.interleaved = interleaved;
    c.units = units;
    const unsigned gb = (unsigned)((units + 255) / 256);
    if (units) (mp::count_launch(), k_outb_dest<<<gb, 256, 0, st>>>(bc, nent, f1, f2));
    scan_u32_to_u64(nent, eoff, units, ntot, tmp, tb, st);
    uint64_t n = 0;
    MP_CUDA(cudaMemcpyAsync(&n, ntot, sizeof n, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    SortBufs sb;
    for (int i = 0; i < 2; i++) {
        sb.lo[i] = arena.alloc<uint64_t>(n + 1);
        sb.id[i] = arena.alloc<uint32_t>(n + 1);
        if (!sb.lo[i] || !sb.id[i]) return set_error(MP_ENOMEM, "device memory for the output entries");
    }
    if (units) (mp::count_launch(), k_out_entries<<<gb, 256, 0, st>>>(c, f1, f2, nent, eoff, sb.lo[0], sb.id[0]));
    int rc = radix_sort(sb, n, false, arena, st, nullptr);
    if (rc) return rc;
    uint64_t *len = arena.alloc<uint64_t>(n + 1);
    plan->val = arena.alloc_persistent<uint32_t>(n + 1);
    plan->off = arena.alloc_persistent<uint64_t>(n + 1);
    size_t tb2 = scan_tmp_bytes(n + 1);
    void *tmp2 = arena.alloc<uint8_t>(tb2);
    if (!len || !plan->val || !plan->off || !tmp2) return set_error(MP_ENOMEM, "device memory for the output offsets");
    const unsigned ge = (unsigned)((n + 255) / 256);
    if (n) (mp::count_launch(), k_out_len<<<ge, 256, 0, st>>>(c, sb.id[sb.cur], n, len, sb.lo[sb.cur], fbytes));
    scan_u64(len, plan->off, n, ntot, tmp2, tb2, st);
    if (n) MP_CUDA(cudaMemcpyAsync(plan->val, sb.id[sb.cur], n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    uint64_t total = 0;
    MP_CUDA(cudaMemcpyAsync(&total, ntot, sizeof total, cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaMemcpyAsync(file_sizes.data(), fbytes, nf * sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
    MP_CUDA(cudaStreamSynchronize(st));
    MP_CUDA(cudaGetLastError());
    plan->n = n;
    plan->total = total;
    plan->rec_start = pr.rec_start;
    plan->interleaved = interleaved;
    return 0;
}

int copy_output_range(const OutputPlan &plan, uint64_t e0, uint64_t e1, const uint8_t *d_fq, uint8_t *dst,
                      cudaStream_t st)
{
    if (e1 <= e0) return 0;
    OutCtx c{};
    c.rec_start = plan.rec_start;
    c.interleaved = plan.interleaved;
    const uint64_t warps = (e1 - e0 + OC_PER_WARP - 1) / OC_PER_WARP;
    (mp::count_launch(), k_out_copy<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, st>>>(
        c, d_fq, plan.val + e0, plan.off + e0, e1 - e0, dst));
    MP_CUDA(cudaGetLastError());
    return 0;
}

int copy_output(const OutputPlan &plan, const uint8_t *d_fq, uint8_t *dst, cudaStream_t st)
{
    return copy_output_range(plan, 0, plan.n, d_fq, dst, st);
}

}  // namespace mp
