// serve.cpp -- request loop with continuous batching over a dsim_batch
// (include/dsim_serve.h).
//
// One worker thread owns the batch.  Each loop: admit pending jobs in arrival
// order while spin slots, job slots and the HBM cap allow (a job that does not
// fit yet waits; smaller jobs behind it may pass), advance every admitted job
// by one quantum (whole chunks, about kQuantumSeconds of device time), then
// read the signals of the jobs that finished, retire them and repack the
// batch so their slots go to the next arrivals.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#pragma GCC visibility push(default)
#include "../../include/dsim_serve.h"
#pragma GCC visibility pop
#include "common.cuh"

namespace {

using Clock = std::chrono::steady_clock;
constexpr double kQuantumSeconds = 0.2;  // device time between admissions

struct Request {
    dsim_job_desc d{};
    std::vector<float> pos, table, grads;
    std::vector<uint8_t> comp;
    std::vector<uint32_t> fiber;
    uint32_t nG = 0;
    uint64_t footprint = 0;
    double tSubmit = 0, tAdmit = -1, tDone = -1;
    uint32_t job = 0;
    bool admitted = false, done = false;
    int status = 0;
    std::vector<double> result;
};

// device bytes a job holds while admitted: two packed buffers of 13 words per
// slot, the sort key, its waveform and the transient signal partials
uint64_t footprint(const dsim_job_desc& d, uint32_t nG) {
    const uint64_t pad = (d.nSpins + 31u) & ~31u;
    return pad * (2 * 13 + 1) * 4 + (uint64_t)d.steps * 4 + 608ull * nG * 15 * 8;
}

}  // namespace

struct dsim_server {
    dsim_batch* b = nullptr;
    int device = 0;
    uint64_t spinCap = 0, hbmCap = 0, hbmSubs = 0, hbmJobs = 0, hbmPeak = 0;
    // device bytes allocated on the first job of a precision form: a mesh's
    // FP64 triangle table (128 B per triangle, per substrate) and the arena's
    // four FP64 fields in both buffers (64 B per spin slot, once)
    std::vector<uint64_t> tri64Bytes;
    std::vector<bool> tri64Held;
    bool fp64Arena = false;
    uint32_t jobCap = 0;
    uint32_t chunk = 20, graphChunks = 8;
    std::mutex mu;
    std::condition_variable cv, doneCv;
    std::deque<uint32_t> pending;
    std::vector<std::unique_ptr<Request>> reqs;
    std::vector<uint32_t> inflight;
    std::thread worker;
    bool started = false, stopping = false;
    Clock::time_point t0;
    double busy = 0, spinSteps = 0, secPerStep = 0;
    uint64_t jobsDone = 0, maxInflight = 0, quanta = 0, compactions = 0, errors = 0;
    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

void worker_loop(dsim_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        // admission (arrival order; a job that does not fit yet waits, smaller ones may pass)
        std::vector<uint32_t> toAdmit;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            if (s->inflight.empty() && s->pending.empty()) {
                if (s->stopping) break;
                s->cv.wait_for(lk, std::chrono::milliseconds(2));
                continue;
            }
            uint64_t used = s->hbmJobs, subs = s->hbmSubs;
            std::vector<bool> held = s->tri64Held;
            bool arena = s->fp64Arena;
            uint64_t slots = 0;
            for (uint32_t t : s->inflight) slots += (s->reqs[t]->d.nSpins + 31u) & ~31u;
            size_t jobs = s->inflight.size();
            for (auto it = s->pending.begin(); it != s->pending.end();) {
                Request& r = *s->reqs[*it];
                const uint64_t pad = (r.d.nSpins + 31u) & ~31u;
                uint64_t extra = 0;
                const bool fp64 = (r.d.flags & (DSIM_JOB_PRECISE | DSIM_JOB_LOCAL)) != 0;
                if (fp64 && !arena) extra += s->spinCap * 64;
                if (fp64 && !held[r.d.substrate]) extra += s->tri64Bytes[r.d.substrate];
                if (subs + extra + used + r.footprint <= s->hbmCap && slots + pad <= s->spinCap && jobs < s->jobCap) {
                    if (fp64) {
                        arena = true;
                        held[r.d.substrate] = true;
                    }
                    subs += extra;
                    used += r.footprint;
                    slots += pad;
                    jobs++;
                    toAdmit.push_back(*it);
                    it = s->pending.erase(it);
                } else {
                    ++it;
                }
            }
            // the precision-form allocations stay for the server's life
            s->hbmSubs = subs;
            s->tri64Held = held;
            s->fp64Arena = arena;
        }
        for (uint32_t t : toAdmit) {
            Request& r = *s->reqs[t];
            r.d.table = r.table.empty() ? nullptr : r.table.data();
            int rc = dsim_batch_submit(s->b, &r.d, r.pos.data(), r.comp.data(),
                                       r.fiber.empty() ? nullptr : r.fiber.data(), &r.job);
            std::lock_guard<std::mutex> lk(s->mu);
            if (rc) {
                r.status = rc;
                r.done = true;
                r.tDone = s->now();
                s->errors++;
                s->doneCv.notify_all();
                continue;
            }
            // the batch holds the job's state on the device now (dsim_batch_submit
            // returns after its uploads): a long stream keeps no host copy of it
            std::vector<float>().swap(r.pos);
            std::vector<uint8_t>().swap(r.comp);
            std::vector<uint32_t>().swap(r.fiber);
            std::vector<float>().swap(r.table);
            r.d.table = nullptr;
            r.admitted = true;
            r.tAdmit = s->now();
            s->hbmJobs += r.footprint;
            if (s->hbmSubs + s->hbmJobs > s->hbmPeak) s->hbmPeak = s->hbmSubs + s->hbmJobs;
            s->inflight.push_back(t);
            if (s->inflight.size() > s->maxInflight) s->maxInflight = s->inflight.size();
        }
        if (s->inflight.empty()) continue;
        // one quantum for every admitted job: whole chunks, about
        // kQuantumSeconds at the last quantum's rate (at most chunk x
        // graphChunks steps), so arrivals wait about that long for admission
        const uint32_t maxSteps = s->chunk * (s->graphChunks ? s->graphChunks : 1);
        uint32_t steps = maxSteps;
        if (s->secPerStep > 0.0) {
            const double whole = std::floor(kQuantumSeconds / s->secPerStep / s->chunk) * s->chunk;
            steps = (uint32_t)std::min<double>(maxSteps, std::max<double>(s->chunk, whole));
        }
        const double ta = s->now();
        int rc = dsim_batch_advance(s->b, steps);
        if (!rc) rc = dsim_batch_sync(s->b);
        const double el = s->now() - ta;
        s->busy += el;
        s->secPerStep = el / steps;
        s->quanta++;
        if (rc) {
            // the device is unusable for this batch: fail every job in flight
            std::lock_guard<std::mutex> lk(s->mu);
            for (uint32_t t : s->inflight) {
                Request& r = *s->reqs[t];
                r.status = rc; r.done = true; r.tDone = s->now();
            }
            s->errors++;
            s->inflight.clear();
            s->doneCv.notify_all();
            continue;
        }
        bool retired = false;
        std::vector<uint32_t> still;
        for (uint32_t t : s->inflight) {
            Request& r = *s->reqs[t];
            uint32_t steps = 0;
            int done = 0;
            if (dsim_batch_job_status(s->b, r.job, &steps, &done) || !done) { still.push_back(t); continue; }
            std::vector<double> out((size_t)15 * r.nG);
            int src = dsim_batch_signal(s->b, r.job, r.grads.data(), r.nG, out.data());
            dsim_batch_retire(s->b, r.job);
            retired = true;
            std::lock_guard<std::mutex> lk(s->mu);
            r.result.swap(out);
            r.status = src;
            r.done = true;
            r.tDone = s->now();
            s->hbmJobs -= r.footprint;
            s->jobsDone++;
            s->spinSteps += (double)r.d.nSpins * (double)r.d.steps;
        }
        if (retired) {
            if (dsim_batch_compact(s->b)) s->errors++;
            s->compactions++;
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->inflight.swap(still);
        }
        s->doneCv.notify_all();
    }
}

}  // namespace

using namespace dsim;

extern "C" {

int dsim_server_create(uint64_t spinCapacity, uint32_t jobCapacity, uint64_t hbmCapBytes, dsim_server** out) {
    if (!out || !spinCapacity || !jobCapacity || !hbmCapBytes) {
        set_last_error(kErrInvalid, "dsim_server_create: bad argument");
        return kErrInvalid;
    }
    *out = nullptr;
    dsim_server* s = new dsim_server();
    cudaGetDevice(&s->device);
    int rc = dsim_batch_create(spinCapacity, jobCapacity, &s->b);
    if (rc) { delete s; return rc; }
    s->spinCap = (spinCapacity + 31) & ~31ull;
    s->jobCap = jobCapacity;
    s->hbmCap = hbmCapBytes;
    *out = s;
    return kOk;
}

void dsim_server_free(dsim_server* s) {
    if (!s) return;
    dsim_server_stop(s);
    dsim_batch_free(s->b);
    delete s;
}

int dsim_server_add_mesh(dsim_server* s, const dsim_mesh* m, uint32_t* sub) {
    if (!s || s->started) { set_last_error(kErrInvalid, "dsim_server_add_mesh: add substrates before start"); return kErrInvalid; }
    int rc = dsim_batch_add_mesh(s->b, m, sub);
    if (rc) return rc;
    uint64_t info[8] = {0};
    if (dsim_mesh_info(m, info) == 0) s->hbmSubs += info[6];
    uint64_t acc[3];
    if (dsim_mesh_accel_info(m, acc) == 0) s->hbmSubs += acc[2];
    s->tri64Bytes.resize(*sub + 1, 0);
    s->tri64Held.resize(*sub + 1, false);
    s->tri64Bytes[*sub] = 128ull * info[1];
    return kOk;
}

int dsim_server_add_cyl(dsim_server* s, const dsim_cyl* c, uint32_t* sub) {
    if (!s || s->started) { set_last_error(kErrInvalid, "dsim_server_add_cyl: add substrates before start"); return kErrInvalid; }
    int rc = dsim_batch_add_cyl(s->b, c, sub);
    if (rc) return rc;
    uint32_t geom[3];
    float L;
    if (dsim_cyl_info(c, geom, &L, nullptr, nullptr, nullptr) == 0)
        s->hbmSubs += (uint64_t)geom[2] * 16 + (uint64_t)geom[0] * geom[0] * geom[0] * (4ull + 4ull * geom[1]);
    s->tri64Bytes.resize(*sub + 1, 0);
    s->tri64Held.resize(*sub + 1, false);
    return kOk;
}

int dsim_server_configure(dsim_server* s, uint32_t chunk, uint32_t occupancy, uint32_t graphChunks) {
    if (!s || s->started) { set_last_error(kErrInvalid, "dsim_server_configure: configure before start"); return kErrInvalid; }
    int rc = dsim_batch_configure(s->b, chunk, occupancy, graphChunks);
    if (rc) return rc;
    s->chunk = chunk;
    s->graphChunks = graphChunks;
    return kOk;
}

int dsim_server_start(dsim_server* s) {
    if (!s || s->started) { set_last_error(kErrInvalid, "dsim_server_start: already started"); return kErrInvalid; }
    s->t0 = Clock::now();
    s->started = true;
    s->worker = std::thread(worker_loop, s);
    return kOk;
}

int dsim_server_submit(dsim_server* s, const dsim_job_desc* d, const float* pos3, const uint8_t* comp,
                       const uint32_t* fiber, const float* gradScaled, uint32_t nG, uint32_t* ticket) {
    if (!s || !d || !pos3 || !comp || !gradScaled || !nG || !ticket || !d->nSpins || !d->steps ||
        (d->waveform == DSIM_WAVE_TABLE && !d->table) || d->substrate >= s->tri64Bytes.size()) {
        set_last_error(kErrInvalid, "dsim_server_submit: bad argument");
        return kErrInvalid;
    }
    std::unique_ptr<Request> r(new Request());
    r->d = *d;
    r->pos.assign(pos3, pos3 + 3 * (size_t)d->nSpins);
    r->comp.assign(comp, comp + d->nSpins);
    if (fiber) r->fiber.assign(fiber, fiber + d->nSpins);
    if (d->waveform == DSIM_WAVE_TABLE) r->table.assign(d->table, d->table + d->steps);
    r->grads.assign(gradScaled, gradScaled + 3 * (size_t)nG);
    r->nG = nG;
    r->footprint = footprint(*d, nG);
    const uint64_t pad = (d->nSpins + 31u) & ~31u;
    std::lock_guard<std::mutex> lk(s->mu);
    // a job that cannot fit even with no other job admitted would wait
    // forever: refused here (a precision-form job also needs the FP64 arena
    // and its mesh's FP64 triangle table, unless they are held already)
    uint64_t need = s->hbmSubs + r->footprint;
    if (d->flags & (DSIM_JOB_PRECISE | DSIM_JOB_LOCAL)) {
        if (!s->fp64Arena) need += s->spinCap * 64;
        if (!s->tri64Held[d->substrate]) need += s->tri64Bytes[d->substrate];
    }
    if (pad > s->spinCap || need > s->hbmCap) {
        set_last_error(kErrTooLarge, "dsim_server_submit: job of %u spins never fits the arena or the HBM cap", d->nSpins);
        return kErrTooLarge;
    }
    r->tSubmit = s->started ? s->now() : 0.0;
    *ticket = (uint32_t)s->reqs.size();
    s->reqs.push_back(std::move(r));
    s->pending.push_back(*ticket);
    s->cv.notify_all();
    return kOk;
}

int dsim_server_poll(dsim_server* s, uint32_t ticket, int* done, double* out, double times[3]) {
    if (!s) return kErrInvalid;
    std::lock_guard<std::mutex> lk(s->mu);
    if (ticket >= s->reqs.size()) { set_last_error(kErrInvalid, "dsim_server_poll: unknown ticket %u", ticket); return kErrInvalid; }
    Request& r = *s->reqs[ticket];
    if (done) *done = r.done ? 1 : 0;
    if (times) { times[0] = r.tSubmit; times[1] = r.tAdmit; times[2] = r.tDone; }
    if (r.done && out && !r.result.empty()) memcpy(out, r.result.data(), r.result.size() * sizeof(double));
    if (r.done && r.status) { set_last_error(r.status, "dsim_server: job %u failed", ticket); return r.status; }
    return kOk;
}

int dsim_server_drain(dsim_server* s) {
    if (!s || !s->started) return kErrInvalid;
    std::unique_lock<std::mutex> lk(s->mu);
    s->doneCv.wait(lk, [&] {
        for (auto& r : s->reqs)
            if (!r->done) return false;
        return true;
    });
    return s->errors ? kErrCuda : kOk;
}

int dsim_server_stop(dsim_server* s) {
    if (!s) return kErrInvalid;
    if (!s->started) return kOk;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
        s->cv.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    s->started = false;
    return kOk;
}

int dsim_server_stats(dsim_server* s, double st[8]) {
    if (!s || !st) return kErrInvalid;
    std::lock_guard<std::mutex> lk(s->mu);
    st[0] = (double)s->jobsDone; st[1] = s->spinSteps; st[2] = s->busy; st[3] = (double)s->maxInflight;
    st[4] = (double)s->hbmPeak; st[5] = (double)s->quanta; st[6] = (double)s->compactions; st[7] = (double)s->errors;
    return kOk;
}

}  // extern "C"
