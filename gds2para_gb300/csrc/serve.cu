// Extraction service: a queue of V0 extraction jobs (each one the work of
// generateStiff + paraGenerator on its own layout) admitted onto the GPU by
// device-memory footprint, each admitted job running on its own host thread
// with its own mesh handle and CUDA stream, so that the kernels of jobs in
// flight overlap on the device.  The reference runs one layout per process
// and has no counterpart.
//
// Admission: while fewer than max_active jobs run, the first queued job
// whose footprint estimate fits the budget minus the estimates of the
// running jobs starts.  A job further back may pass one that does not fit
// yet, but only 2 * max_active times: after that the bypassed job holds the
// queue until it fits.  A job that fits no budget runs alone.  The estimate
// is a size model (edges, nodes, right-hand sides, Krylov restart) scaled by
// the largest ratio of measured pool high-water to estimate seen on jobs that
// ran alone.  A job whose estimate with all ports in one block exceeds the
// budget runs its ports in the widest power-of-two blocks that fit.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

using namespace g2p;

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// Host copy of a g2p_mesh_desc (arrays may have been host or device memory).
struct DescCopy {
    g2p_mesh_desc d{};
    std::vector<double> xn, yn, zn, epsn, sign, area;
    std::vector<int64_t> mark_node, mark_edge, edge_ptr, edges;
    std::vector<int32_t> mark_port, side_ptr, dir;
    std::vector<uint8_t> cdt_return;
};

template <class T>
g2p_status fetch(std::vector<T> &dst, const T *src, int64_t n) {
    dst.resize((size_t)std::max<int64_t>(n, 0));
    if (n > 0) {
        if (!src) { set_last_message("missing mesh array"); return G2P_ERR_INVALID; }
        G2P_CUDA(cudaMemcpy(dst.data(), src, sizeof(T) * n, cudaMemcpyDefault));
    }
    return G2P_OK;
}

g2p_status copy_desc(const g2p_mesh_desc *in, DescCopy &c) {
    if (!in) { set_last_message("null mesh description"); return G2P_ERR_INVALID; }
    if (in->nx < 3 || in->ny < 3 || in->nz < 3 || in->num_ports < 0 || in->num_cdt < 1) {
        set_last_message("invalid mesh description");
        return G2P_ERR_INVALID;
    }
    Dims d;
    d.init(in->nx, in->ny, in->nz);
    c.d = *in;
    G2P_TRY(fetch(c.xn, in->xn, d.nx)); G2P_TRY(fetch(c.yn, in->yn, d.ny)); G2P_TRY(fetch(c.zn, in->zn, d.nz));
    G2P_TRY(fetch(c.epsn, in->stack_epsn, d.nz)); G2P_TRY(fetch(c.sign, in->stack_sign, d.nz));
    G2P_TRY(fetch(c.mark_node, in->mark_node, d.N_node)); G2P_TRY(fetch(c.mark_edge, in->mark_edge, d.N_edge));
    G2P_TRY(fetch(c.mark_port, in->mark_port, in->num_cdt)); G2P_TRY(fetch(c.cdt_return, in->cdt_return, in->num_cdt));
    G2P_TRY(fetch(c.side_ptr, in->port_side_ptr, (int64_t)in->num_ports + 1));
    const int64_t nsides = in->num_ports > 0 ? c.side_ptr[in->num_ports] : 0;
    G2P_TRY(fetch(c.edge_ptr, in->side_edge_ptr, nsides + 1));
    const int64_t nedges = nsides > 0 ? c.edge_ptr[nsides] : 0;
    G2P_TRY(fetch(c.edges, in->side_edges, nedges));
    G2P_TRY(fetch(c.area, in->side_area, nsides));
    G2P_TRY(fetch(c.dir, in->side_dir, nsides));
    c.d.xn = c.xn.data(); c.d.yn = c.yn.data(); c.d.zn = c.zn.data();
    c.d.stack_epsn = c.epsn.data(); c.d.stack_sign = c.sign.data();
    c.d.mark_node = c.mark_node.data(); c.d.mark_edge = c.mark_edge.data();
    c.d.mark_port = c.mark_port.data(); c.d.cdt_return = c.cdt_return.data();
    c.d.port_side_ptr = c.side_ptr.data(); c.d.side_edge_ptr = c.edge_ptr.data();
    c.d.side_edges = c.edges.data(); c.d.side_area = c.area.data(); c.d.side_dir = c.dir.data();
    return G2P_OK;
}

// Size model of one job's device memory (bytes): mesh arrays, S and the V0
// bases per edge; Laplacians, AMG levels and the Krylov blocks per node and
// right-hand side.
double size_model(const g2p_mesh_desc &in, const g2p_solver_params &p) {
    Dims d;
    d.init(in.nx, in.ny, in.nz);
    const int P = std::max(1, in.num_ports);
    const int k = p.batch == 0 ? 1 : std::min(p.batch >= 2 ? p.batch : P, std::min(P, 256));
    const int m = p.restart > 0 ? std::min(p.restart, 64) : 30;
    const int mi = p.inner_restart > 0 ? std::min(p.inner_restart, 64) : m;
    const double per_edge = 4 + 4 + 1 + 40 + 13 * 12.0 + 8;          // marks, map, flags, edge views, S
    const double per_node = 2 * 7 * 12.0 * 2.5;                        // Ad copies over the AMG levels
    // Krylov basis (V and Z) and work vectors per right-hand side and node
    const double per_rhs = p.precision == G2P_PREC_MIXED ? (2 * mi + 9) * 4.0 + 6 * 8.0 : (2 * m + 9) * 8.0;
    return d.N_edge * per_edge + d.N_node * per_node + (double)d.N_node * k * per_rhs;
}

struct Job {
    int64_t id = 0;
    DescCopy desc;
    g2p_solver_params params{};
    double model = 0, estimate = 0;     // size model; model x scale at admission
    Clock::time_point t_submit, t_start, t_end;
    bool started = false, done = false, solo = false;
    int64_t start_seq = 0;
    g2p_status status = G2P_OK;
    std::string error;
    std::vector<double> z;
    g2p_extract_stats stats{};
    uint64_t measured = 0;
    int bypassed = 0;                   // times a later job started ahead of it
};

// The port block width a job runs with: its own setting, narrowed to the
// widest power-of-two block whose estimate fits the budget.
int32_t fitting_batch(const g2p_mesh_desc &d, g2p_solver_params p, double scale, double budget) {
    const int P = std::max(1, d.num_ports);
    if (p.batch == 0 || size_model(d, p) * scale <= budget) return p.batch;
    int w = 1;
    while (w * 2 < P) w *= 2;
    for (; w >= 2; w /= 2) {
        p.batch = w;
        if (size_model(d, p) * scale <= budget) return w;
    }
    return 0;          // one port at a time
}

}  // namespace

struct g2p_server {
    int device = 0;
    int64_t budget = 0;
    int max_active = 1;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<std::shared_ptr<Job>> queue;
    std::map<int64_t, std::shared_ptr<Job>> jobs;
    std::vector<std::thread> workers;
    std::thread dispatcher;
    int active = 0;
    double committed = 0;      // estimates of the running jobs
    double scale = 1.0;        // measured / model, from jobs that ran alone
    int64_t next_id = 1;
    int64_t starts = 0;        // jobs started so far
    bool stopping = false;

    void run_job(std::shared_ptr<Job> job);
    void dispatch_loop();
};

void g2p_server::run_job(std::shared_ptr<Job> job) {
    cudaSetDevice(device);
    cudaMemPool_t pool = nullptr;
    if (job->solo && cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t zero = 0;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero);
    }
    g2p_mesh *h = nullptr;
    g2p_status st = g2p_mesh_create(&job->desc.d, &h);
    if (st == G2P_OK) {
        int64_t leng = 0;
        st = g2p_generate_stiff(h, &leng);
    }
    if (st == G2P_OK) {
        const int P = job->desc.d.num_ports;
        job->z.assign((size_t)2 * job->desc.d.nfreq * P * P, 0.0);
        st = g2p_para_generator(h, &job->params, job->z.data(), &job->stats);
    }
    if (st != G2P_OK) job->error = g2p_last_error();
    if (h) g2p_mesh_destroy(h);
    if (pool && job->solo) {
        uint64_t hi = 0;
        if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &hi) == cudaSuccess) job->measured = hi;
    }
    std::lock_guard<std::mutex> lock(mu);
    job->status = st;
    job->t_end = Clock::now();
    job->done = true;
    // alone for its whole run: alone at its start and nothing started since
    job->solo = job->solo && starts == job->start_seq;
    if (!job->solo) job->measured = 0;
    active--;
    committed -= job->estimate;
    if (job->solo && job->measured > 0) {
        if (job->model > 0) scale = std::max(scale, (double)job->measured / job->model);
    }
    cv.notify_all();
}

void g2p_server::dispatch_loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lock(mu);
    const int max_bypass = 2 * max_active;
    size_t pick = 0;
    // the queue position of the job to start now, or queue.size() for none
    auto admissible = [&]() -> size_t {
        if (queue.empty() || active >= max_active) return queue.size();
        for (size_t i = 0; i < queue.size(); i++) {
            const Job &q = *queue[i];
            const double est = size_model(q.desc.d, q.params) * scale;
            if (active == 0 || committed + est <= (double)budget) return i;
            if (q.bypassed >= max_bypass) break;      // it holds the queue until it fits
        }
        return queue.size();
    };
    for (;;) {
        cv.wait(lock, [&] {
            if (stopping && queue.empty()) return true;
            pick = admissible();
            return pick < queue.size();
        });
        if (stopping && queue.empty()) return;
        std::shared_ptr<Job> job = queue[pick];
        for (size_t i = 0; i < pick; i++) queue[i]->bypassed++;
        queue.erase(queue.begin() + (std::ptrdiff_t)pick);
        job->model = size_model(job->desc.d, job->params);
        job->estimate = job->model * scale;
        job->solo = active == 0;
        job->start_seq = ++starts;
        job->started = true;
        job->t_start = Clock::now();
        active++;
        committed += job->estimate;
        workers.emplace_back([this, job] { run_job(job); });
    }
}

extern "C" g2p_status g2p_server_create(int64_t mem_budget_bytes, int32_t max_active, g2p_server **out) {
    if (!out || max_active < 1 || mem_budget_bytes <= 0) {
        set_last_message("g2p_server_create: need a positive budget and max_active >= 1");
        return G2P_ERR_INVALID;
    }
    auto *s = new g2p_server();
    G2P_CUDA(cudaGetDevice(&s->device));
    retain_pool_memory(s->device);
    s->budget = mem_budget_bytes;
    s->max_active = max_active;
    s->dispatcher = std::thread([s] { s->dispatch_loop(); });
    *out = s;
    return G2P_OK;
}

extern "C" g2p_status g2p_server_submit(g2p_server *s, const g2p_mesh_desc *desc, const g2p_solver_params *p,
                                        int64_t *job_id) {
    if (!s || !job_id) { set_last_message("null argument"); return G2P_ERR_INVALID; }
    auto job = std::make_shared<Job>();
    G2P_TRY(copy_desc(desc, job->desc));
    if (p) job->params = *p;
    else g2p_default_params(&job->params, 0);
    std::lock_guard<std::mutex> lock(s->mu);
    // fixed margin, not the measured scale: a job's block width (and so its
    // result) depends only on its own description and the budget
    job->params.batch = fitting_batch(job->desc.d, job->params, 1.5, (double)s->budget);
    if (s->stopping) { set_last_message("server is shutting down"); return G2P_ERR_STATE; }
    // a job whose estimate exceeds the budget is still run, alone
    job->id = s->next_id++;
    job->t_submit = Clock::now();
    s->jobs[job->id] = job;
    s->queue.push_back(job);
    s->cv.notify_all();
    *job_id = job->id;
    return G2P_OK;
}

extern "C" g2p_status g2p_server_wait(g2p_server *s, int64_t job_id, double *z_out, g2p_extract_stats *st,
                                      g2p_job_times *t) {
    if (!s) { set_last_message("null server"); return G2P_ERR_INVALID; }
    std::shared_ptr<Job> job;
    {
        std::unique_lock<std::mutex> lock(s->mu);
        auto it = s->jobs.find(job_id);
        if (it == s->jobs.end()) { set_last_message("unknown job %lld", (long long)job_id); return G2P_ERR_INVALID; }
        job = it->second;
        s->cv.wait(lock, [&] { return job->done; });
        s->jobs.erase(it);
    }
    if (job->status != G2P_OK && job->status != G2P_ERR_NOT_CONVERGED) {
        set_last_message("job %lld: %s", (long long)job_id, job->error.c_str());
        return job->status;
    }
    if (z_out && !job->z.empty()) memcpy(z_out, job->z.data(), sizeof(double) * job->z.size());
    if (st) *st = job->stats;
    if (t) {
        t->queued_ms = ms_between(job->t_submit, job->t_start);
        t->run_ms = ms_between(job->t_start, job->t_end);
        t->total_ms = ms_between(job->t_submit, job->t_end);
        t->footprint_estimate = (int64_t)job->estimate;
        t->footprint_measured = (int64_t)job->measured;
        t->ran_alone = job->solo ? 1 : 0;
    }
    return job->status;
}

extern "C" g2p_status g2p_server_destroy(g2p_server *s) {
    if (!s) return G2P_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stopping = true;
        s->cv.notify_all();
    }
    if (s->dispatcher.joinable()) s->dispatcher.join();
    for (auto &w : s->workers)
        if (w.joinable()) w.join();
    delete s;
    return G2P_OK;
}
