// serve.cu -- the serving loop: continuous batching of many tenants'
// alloc / free / fetch requests over one resident pool and buffer manager.
//
// No reference counterpart (the reference has batch drivers only).  Requests
// replay in real time from their arrival stamps.  Each tenant owns a ring of
// page slots in device memory: ALLOC n appends n new pages, FREE n releases
// min(n, pages the tenant holds) of its oldest pages, FETCH n pins and then
// releases n pages of a shared fetch trace in the buffer manager.
//
// Admission is by free-page budget, shared by the whole pool: the pages free
// below max_occupancy when the server is created.  An ALLOC is admitted when
// the pages the tenants hold on the device (counting allocations in flight,
// and frees only once their batch has finished) plus its own fit the budget;
// otherwise it waits at the front of its tenant's queue until frees land.
// Only an ALLOC that could never fit (more pages than the budget, the
// tenant's ring or its optional quota) is rejected.  A tenant's ALLOCs keep
// their arrival order; a later FREE may pass a waiting ALLOC when every page
// it releases is older than that ALLOC (so it releases exactly the pages it
// would in arrival order), and a FETCH may always pass.  A FREE waits until
// the pages it releases have been allocated on the device.  Admitted
// requests of all tenants form the next batch as soon as one of n_streams
// batch slots is free, so batches overlap on the device and requests that
// arrive while others run join the following batch.  Bitmap, clock hands,
// rings and RNG streams stay resident between batches.
//
// Results: a request's status and page count depend only on its tenant's
// own requests, so they are the same alone and in a mix for every request
// the mix admits.  Contention changes when a request is admitted (its
// latency), not what it gets.  The one exception: when no arrivals are left,
// nothing is in flight and nothing can be admitted, the loop stops and the
// requests still waiting end with status -1 (they waited for memory that no
// remaining request frees); a tenant alone would have had that memory.
#include <algorithm>
#include <chrono>
#include <deque>
#include <new>
#include <vector>

#include "internal.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Pending {
    uint64_t req;
    uint64_t pages;
    bool done;
};

struct Tenant {
    uint64_t head = 0, tail = 0, completed = 0;   // ring positions (monotone)
    uint64_t logical = 0;                         // pages held after the admitted requests
    std::deque<Pending> allocs;                   // admitted allocations, admission order
    std::deque<uint64_t> queue;                   // arrived, not yet admitted (arrival order)
};

struct BatchSlot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    uint64_t freed_pages = 0;        // pages the batch releases (back in the budget when it finishes)
    pbm_group* h_groups = nullptr;   // pinned
    pbm_group* d_groups = nullptr;
    int32_t* d_frames = nullptr;
    std::vector<uint64_t> reqs;
    uint32_t n_groups = 0;
};

}  // namespace

struct pbm_server {
    pbm_pool* pool;
    pbm_bufmgr* bm;
    const int32_t* d_fetch_pages;
    uint64_t n_fetch_pages;
    pbm_server_config cfg;
    int32_t* d_rings;
    int32_t* d_identity;             // 0, 1, 2, ... (release lists of fetch batches)
    std::vector<BatchSlot> slots;
    uint32_t max_groups;
    uint32_t max_fetch;
    uint64_t n_pages;
    uint64_t budget;                 // pages the tenants may hold together
    uint64_t quota;                  // pages one tenant may hold (UINT64_MAX: no per-tenant cap)
    uint64_t device_held;            // pages held or being allocated on the device by the tenants
    uint32_t seed;
    uint64_t fetch_cursor;
    std::vector<Tenant> tenants;
};

extern "C" {

int pbm_server_create(pbm_pool* pool, pbm_bufmgr* bm, const int32_t* d_fetch_pages, uint64_t n_fetch_pages,
                      const pbm_server_config* cfg, pbm_server** out) {
    PBM_ON_POOL_DEVICE(pool);
    if (!pool || !cfg || !out || cfg->n_tenants == 0 || cfg->ring_pages == 0 || cfg->n_streams == 0 ||
        cfg->max_batch_requests == 0 || cfg->max_batch_requests > 2048 || !(cfg->max_occupancy > 0.0) ||
        cfg->max_occupancy > 1.0)
        return PBM_ERR_INVALID;
    if (bm && (!d_fetch_pages || n_fetch_pages == 0)) return PBM_ERR_INVALID;
    *out = nullptr;
    pbm_server* s = new (std::nothrow) pbm_server();
    if (!s) return PBM_ERR_NOMEM;
    s->pool = pool;
    s->bm = bm;
    s->d_fetch_pages = d_fetch_pages;
    s->n_fetch_pages = n_fetch_pages;
    s->cfg = *cfg;
    s->max_groups = 2u * cfg->max_batch_requests;
    s->max_fetch = cfg->max_fetch_pages ? cfg->max_fetch_pages : (1u << 22);
    s->n_pages = pool->n_pages;
    s->seed = 0x51u;
    s->fetch_cursor = 0;
    s->tenants.resize(cfg->n_tenants);
    {
        uint64_t used = 0;
        if (pbm_pool_used(pool, &used, nullptr) != PBM_OK) { delete s; return PBM_ERR_CUDA; }
        const uint64_t cap = (uint64_t)(cfg->max_occupancy * (double)pool->n_pages);
        s->budget = cap > used ? cap - used : 0;
    }
    s->quota = cfg->tenant_quota_pages ? cfg->tenant_quota_pages : UINT64_MAX;
    s->device_held = 0;
    const size_t ring_total = (size_t)cfg->n_tenants * cfg->ring_pages;
    bool ok = cudaMalloc(&s->d_rings, ring_total * sizeof(int32_t)) == cudaSuccess &&
              cudaMemset(s->d_rings, 0xff, ring_total * sizeof(int32_t)) == cudaSuccess &&
              cudaMalloc(&s->d_identity, (size_t)s->max_fetch * sizeof(int32_t)) == cudaSuccess;
    if (ok) {
        std::vector<int32_t> id(s->max_fetch);
        for (uint32_t i = 0; i < s->max_fetch; ++i) id[i] = (int32_t)i;
        ok = cudaMemcpy(s->d_identity, id.data(), id.size() * 4, cudaMemcpyHostToDevice) == cudaSuccess;
    }
    s->slots.resize(cfg->n_streams);
    for (auto& b : s->slots) {
        if (!ok) break;
        ok = cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming) == cudaSuccess &&
             cudaMallocHost(&b.h_groups, s->max_groups * sizeof(pbm_group)) == cudaSuccess &&
             cudaMalloc(&b.d_groups, s->max_groups * sizeof(pbm_group)) == cudaSuccess &&
             (!bm || cudaMalloc(&b.d_frames, (size_t)s->max_fetch * sizeof(int32_t)) == cudaSuccess);
    }
    if (!ok) {
        cudaGetLastError();
        pbm_server_destroy(s);
        return PBM_ERR_NOMEM;
    }
    *out = s;
    return PBM_OK;
}

int pbm_server_destroy(pbm_server* s) {
    if (!s) return PBM_ERR_INVALID;
    pbm::DeviceScope scope(s->pool->device);
    for (auto& b : s->slots) {
        if (b.stream) cudaStreamSynchronize(b.stream);
        if (b.stream) cudaStreamDestroy(b.stream);
        if (b.done) cudaEventDestroy(b.done);
        cudaFreeHost(b.h_groups);
        cudaFree(b.d_groups);
        cudaFree(b.d_frames);
    }
    cudaFree(s->d_rings);
    cudaFree(s->d_identity);
    delete s;
    return PBM_OK;
}

int pbm_server_run(pbm_server* s, const pbm_request* reqs, uint64_t n, pbm_request_result* res,
                   pbm_server_report* report) {
    if (!s || (n && (!reqs || !res))) return PBM_ERR_INVALID;
    pbm::DeviceScope scope(s->pool->device);
    for (uint64_t i = 0; i < n; ++i) {
        if (reqs[i].tenant >= s->cfg.n_tenants || reqs[i].op < PBM_REQ_ALLOC || reqs[i].op > PBM_REQ_FETCH)
            return PBM_ERR_INVALID;
        if (reqs[i].op == PBM_REQ_FETCH && (!s->bm || reqs[i].count > s->max_fetch)) return PBM_ERR_INVALID;
        if (i && reqs[i].arrival_s < reqs[i - 1].arrival_s) return PBM_ERR_INVALID;
        res[i] = pbm_request_result{};
        res[i].status = -1;
    }
    int rc = PBM_OK;
    const uint32_t R = s->cfg.ring_pages;
    const auto t0 = Clock::now();
    auto now_s = [&]() { return std::chrono::duration<double>(Clock::now() - t0).count(); };
    uint64_t next = 0, finished = 0, batches = 0, in_flight = 0, max_in_flight = 0, batch_reqs = 0;
    uint64_t pages_done = 0, waited = 0, idle_passes = 0;
    std::vector<uint8_t> waited_flag(n, 0), free_sized(n, 0), fully_admitted(n, 0);
    std::vector<uint32_t> parts_pending(n, 0);
    std::vector<uint64_t> free_done(n, 0);
    const double give_up_s = (n ? reqs[n - 1].arrival_s : 0.0) + s->cfg.drain_timeout_s;
    uint32_t rr = 0;   // round-robin start tenant
    while (finished < n) {
        const double t = now_s();
        // arrivals
        while (next < n && reqs[next].arrival_s <= t) {
            s->tenants[reqs[next].tenant].queue.push_back(next);
            ++next;
        }
        // completions
        for (auto& b : s->slots) {
            if (!b.busy) continue;
            cudaError_t q = cudaEventQuery(b.done);
            if (q == cudaErrorNotReady) continue;
            if (q != cudaSuccess) return PBM_ERR_CUDA;
            const double td = now_s();
            for (uint64_t r : b.reqs) {
                Tenant& tn = s->tenants[reqs[r].tenant];
                if (reqs[r].op == PBM_REQ_ALLOC) {
                    for (auto& p : tn.allocs) if (p.req == r) p.done = true;
                    while (!tn.allocs.empty() && tn.allocs.front().done) {
                        tn.completed += tn.allocs.front().pages;
                        tn.allocs.pop_front();
                    }
                }
                // a FREE split over several batches is done with its last part
                if (--parts_pending[r] != 0 || !fully_admitted[r]) continue;
                res[r].done_s = td;
                res[r].status = 0;
                pages_done += res[r].pages;
                ++finished;
            }
            s->device_held -= b.freed_pages;   // the batch's frees have landed
            b.freed_pages = 0;
            b.reqs.clear();
            b.busy = false;
            --in_flight;
        }
        // admission into a free batch slot
        BatchSlot* slot = nullptr;
        for (auto& b : s->slots) if (!b.busy) { slot = &b; break; }
        if (slot) {
            uint32_t ng = 0, nreq = 0;
            uint64_t fetch_pages = 0;
            const uint64_t fetch_begin = s->fetch_cursor;
            const double ta = now_s();
            for (uint32_t k = 0; k < s->cfg.n_tenants && nreq < s->cfg.max_batch_requests; ++k) {
                const uint32_t ti = (rr + k) % s->cfg.n_tenants;
                Tenant& tn = s->tenants[ti];
                uint64_t virt = tn.logical;    // pages held after the earlier queued requests, in arrival order
                bool alloc_waits = false;      // an earlier ALLOC of this tenant waits for memory
                size_t qi = 0;
                while (qi < tn.queue.size() && nreq < s->cfg.max_batch_requests && ng + 2u <= s->max_groups) {
                    const uint64_t r = tn.queue[qi];
                    const pbm_request& q = reqs[r];
                    if (q.op == PBM_REQ_ALLOC) {
                        if (alloc_waits) {     // ALLOCs keep their order
                            virt += q.count;
                            ++qi;
                            continue;
                        }
                        if (q.count > s->budget || q.count > R || q.count > s->quota) {   // can never fit
                            res[r].status = PBM_ERR_EXHAUSTED;
                            res[r].admit_s = res[r].done_s = ta;
                            res[r].pages = 0;
                            tn.queue.erase(tn.queue.begin() + (std::ptrdiff_t)qi);
                            ++finished;
                            continue;
                        }
                        if (s->device_held + q.count > s->budget || tn.logical + q.count > R ||
                            tn.logical + q.count > s->quota) {   // waits until frees land
                            if (!waited_flag[r]) { waited_flag[r] = 1; ++waited; }
                            alloc_waits = true;
                            virt += q.count;
                            ++qi;
                            continue;
                        }
                        const uint64_t pos = tn.tail % R;
                        const uint64_t first = std::min<uint64_t>(q.count, R - pos);
                        slot->h_groups[ng++] = pbm_group{PBM_OP_ALLOC, (uint32_t)first, (uint64_t)ti * R + pos};
                        if (q.count > first)
                            slot->h_groups[ng++] = pbm_group{PBM_OP_ALLOC, (uint32_t)(q.count - first), (uint64_t)ti * R};
                        tn.tail += q.count;
                        tn.logical += q.count;
                        virt += q.count;
                        s->device_held += q.count;
                        tn.allocs.push_back(Pending{r, q.count, false});
                        res[r].pages = q.count;
                        fully_admitted[r] = 1;
                    } else if (q.op == PBM_REQ_FREE) {
                        // its size follows from the tenant's own earlier requests: fixed when first seen
                        if (!free_sized[r]) {
                            free_sized[r] = 1;
                            res[r].pages = std::min<uint64_t>(q.count, virt);
                        }
                        const uint64_t left = res[r].pages - free_done[r];
                        virt -= left;
                        // pages it may release now: held (older than any waiting ALLOC) and
                        // allocated on the device; the rest waits for the ALLOCs that bring them
                        const uint64_t part = std::min<uint64_t>(left, std::min<uint64_t>(tn.logical,
                                                                                         tn.completed - tn.head));
                        if (part) {
                            const uint64_t pos = tn.head % R;
                            const uint64_t first = std::min<uint64_t>(part, R - pos);
                            slot->h_groups[ng++] = pbm_group{PBM_OP_FREE, (uint32_t)first, (uint64_t)ti * R + pos};
                            if (part > first)
                                slot->h_groups[ng++] = pbm_group{PBM_OP_FREE, (uint32_t)(part - first), (uint64_t)ti * R};
                            tn.head += part;
                            tn.logical -= part;
                            free_done[r] += part;
                            slot->freed_pages += part;
                            if (res[r].admit_s == 0.0) res[r].admit_s = ta;
                            slot->reqs.push_back(r);
                            ++parts_pending[r];
                            ++nreq;
                        }
                        if (free_done[r] < res[r].pages) break;   // the rest waits; so do later requests
                        fully_admitted[r] = 1;
                        if (!part) {   // nothing to release (a FREE of 0 pages): done with the batch
                            if (res[r].admit_s == 0.0) res[r].admit_s = ta;
                            slot->reqs.push_back(r);
                            ++parts_pending[r];
                            ++nreq;
                        }
                        tn.queue.erase(tn.queue.begin() + (std::ptrdiff_t)qi);
                        continue;
                    } else {
                        if (fetch_pages + q.count > s->max_fetch) break;
                        fetch_pages += q.count;
                        res[r].pages = q.count;
                        fully_admitted[r] = 1;
                    }
                    res[r].admit_s = ta;
                    slot->reqs.push_back(r);
                    ++parts_pending[r];
                    tn.queue.erase(tn.queue.begin() + (std::ptrdiff_t)qi);
                    ++nreq;
                }
            }
            rr = (rr + 1u) % s->cfg.n_tenants;
            if (nreq) {
                cudaStream_t st = slot->stream;
                if (ng <= PBM_MAX_INLINE_GROUPS) {
                    // the batch's table rides in the launch: no copy ahead of it
                    if (ng) rc = pbm_batch_launch(s->pool, &s->cfg.walk, nullptr, slot->h_groups, ng, s->d_rings,
                                                  (uint64_t)s->cfg.n_tenants * R, s->seed++, nullptr,
                                                  PBM_LAUNCH_PERSISTENT, st);
                    if (rc) return rc;
                } else {
                    PBM_CUDA_TRY(cudaMemcpyAsync(slot->d_groups, slot->h_groups, ng * sizeof(pbm_group),
                                                 cudaMemcpyHostToDevice, st));
                    rc = pbm_batch_launch(s->pool, &s->cfg.walk, slot->d_groups, nullptr, ng, s->d_rings,
                                          (uint64_t)s->cfg.n_tenants * R, s->seed++, nullptr, PBM_LAUNCH_PERSISTENT, st);
                    if (rc) return rc;
                }
                if (fetch_pages) {
                    // the batch's fetches read the trace from fetch_begin (wrapping), pin, then release
                    uint64_t done_f = 0;
                    while (done_f < fetch_pages) {
                        const uint64_t pos = (fetch_begin + done_f) % s->n_fetch_pages;
                        const uint64_t len = std::min<uint64_t>(fetch_pages - done_f, s->n_fetch_pages - pos);
                        rc = pbm_bufmgr_round(s->bm, nullptr, nullptr, 0, s->d_fetch_pages + pos, (uint32_t)len,
                                              (uint32_t)(fetch_begin + done_f), slot->d_frames + done_f, 0, st);
                        if (rc) return rc;
                        done_f += len;
                    }
                    rc = pbm_bufmgr_round(s->bm, slot->d_frames, s->d_identity, (uint32_t)fetch_pages, nullptr, 0, 0,
                                          nullptr, 0, st);
                    if (rc) return rc;
                    s->fetch_cursor = (fetch_begin + fetch_pages) % s->n_fetch_pages;
                }
                PBM_CUDA_TRY(cudaEventRecord(slot->done, st));
                const double tl = now_s();
                for (uint64_t r : slot->reqs) res[r].launch_s = tl;
                slot->busy = true;
                ++batches;
                batch_reqs += nreq;
                ++in_flight;
                max_in_flight = std::max(max_in_flight, in_flight);
                continue;
            }
        }
        // nothing left to arrive, nothing in flight, and this pass admitted
        // nothing: no later pass can admit anything either (stranded requests)
        if (next >= n && in_flight == 0 && finished < n) {
            ++idle_passes;
            if (idle_passes > 1 || now_s() > give_up_s) break;
        } else {
            idle_passes = 0;
        }
    }
    for (auto& b : s->slots) cudaStreamSynchronize(b.stream);
    if (report) {
        std::vector<double> lat;
        lat.reserve(n);
        uint64_t rejected = 0;
        for (uint64_t i = 0; i < n; ++i) {
            if (res[i].status != 0) { ++rejected; continue; }
            res[i].latency_s = res[i].done_s - reqs[i].arrival_s;
            lat.push_back(res[i].latency_s);
        }
        std::sort(lat.begin(), lat.end());
        auto pct = [&](double p) {
            if (lat.empty()) return 0.0;
            size_t k = (size_t)std::min<double>((double)lat.size() - 1.0, p * (double)(lat.size() - 1) + 0.5);
            return lat[k];
        };
        report->requests = n;
        report->completed = finished;
        report->rejected = rejected;
        report->pages = pages_done;
        report->batches = batches;
        report->max_in_flight = max_in_flight;
        report->wall_s = now_s();
        report->p50_s = pct(0.50);
        report->p99_s = pct(0.99);
        report->mean_batch_requests = batches ? (double)batch_reqs / (double)batches : 0.0;
        report->waited = waited;
        uint64_t stranded = 0;
        for (uint64_t i = 0; i < n; ++i) stranded += res[i].status == -1;
        report->stranded = stranded;
    }
    // stranded requests (nothing could ever admit them) end the run normally;
    // only running out of drain_timeout_s with work still possible is a timeout
    return (finished == n || idle_passes > 1) ? PBM_OK : PBM_ERR_TIMEOUT;
}

int pbm_server_tenant_pages(pbm_server* s, uint32_t tenant, int32_t* h_out, uint64_t max_out, uint64_t* h_n) {
    if (!s || tenant >= s->cfg.n_tenants || !h_n) return PBM_ERR_INVALID;
    pbm::DeviceScope scope(s->pool->device);
    const Tenant& tn = s->tenants[tenant];
    const uint64_t k = tn.tail - tn.head;
    *h_n = k;
    if (!h_out) return PBM_OK;
    if (max_out < k) return PBM_ERR_INVALID;
    const uint32_t R = s->cfg.ring_pages;
    const int32_t* ring = s->d_rings + (size_t)tenant * R;
    const uint64_t pos = tn.head % R;
    const uint64_t first = std::min<uint64_t>(k, R - pos);
    PBM_CUDA_TRY(cudaDeviceSynchronize());
    PBM_CUDA_TRY(cudaMemcpy(h_out, ring + pos, first * 4, cudaMemcpyDeviceToHost));
    if (k > first) PBM_CUDA_TRY(cudaMemcpy(h_out + first, ring, (k - first) * 4, cudaMemcpyDeviceToHost));
    return PBM_OK;
}

}  // extern "C"
