// lbm_batch.cu -- ensembles of independent lid-driven cavities on one GPU.
//
// An ensemble holds any number of cavities (lattices) of different sizes,
// parameters, storage types and step counts, each with its own step
// counter.  A tick advances every active cavity by k steps with one launch
// per storage group and step (k_step / k_step2: each block reads its
// cavity's parity from the descriptor table), pairs of steps replayed from a
// captured CUDA graph.  With kernel shape 3 a chunk of 16-bit cavities whose
// members are all at an alpha step runs the staged-tile kernel instead, and
// so do beta steps of the cavities whose rows are whole 16-byte units (they
// form their own groups).  The static batch (lbm_cu_batch_*) runs a fixed
// ensemble to completion; the server (lbm_cu_server_*) admits queued solves
// between ticks under an HBM budget and retires finished ones (continuous
// batching).  Results of a cavity do not depend on the other members of its
// ensemble: every cavity is computed by the same per-cell arithmetic as a
// lone lattice.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <memory>
#include <string>
#include <vector>

#include "lbm_internal.h"

using namespace lbm;
using namespace lbm_rt;

namespace lbm_rt {

template <typename S, bool PAIR>
int launch_tick_t(bool les, const BatchArgs &a, int blocks, int j, int uni, cudaStream_t st) {
    if (blocks <= 0) return 0;
    if constexpr (PAIR) {
        if (les) k_step2<S, true><<<blocks, kBlock, 0, st>>>(a, j);
        else k_step2<S, false><<<blocks, kBlock, 0, st>>>(a, j);
    } else if constexpr (sizeof(S) >= 4) {
        // float and double chunks whose cavities are all at the same kind of
        // step run that kind's kernel alone (its own launch bounds)
        if (uni == 1) {
            if (les) k_step<S, true, 1><<<blocks, kBlock, 0, st>>>(a, j);
            else k_step<S, false, 1><<<blocks, kBlock, 0, st>>>(a, j);
        } else if (uni == 2) {
            if (les) k_step<S, true, 2><<<blocks, kBlock, 0, st>>>(a, j);
            else k_step<S, false, 2><<<blocks, kBlock, 0, st>>>(a, j);
        } else {
            if (les) k_step<S, true><<<blocks, kBlock, 0, st>>>(a, j);
            else k_step<S, false><<<blocks, kBlock, 0, st>>>(a, j);
        }
    } else {
        (void)uni;
        if (les) k_step<S, true><<<blocks, kBlock, 0, st>>>(a, j);
        else k_step<S, false><<<blocks, kBlock, 0, st>>>(a, j);
    }
    CU(cudaGetLastError());
    return 0;
}

int launch_tick(int storage, bool pair, bool les, const BatchArgs &a, int blocks, int j, int uni, cudaStream_t st) {
    if (pair) {
        switch (storage) {
            case kF32: return launch_tick_t<float, true>(les, a, blocks, j, uni, st);
            case kF16: return launch_tick_t<__half, true>(les, a, blocks, j, uni, st);
            case kBF16: return launch_tick_t<__nv_bfloat16, true>(les, a, blocks, j, uni, st);
            case kC16: return launch_tick_t<c16_t, true>(les, a, blocks, j, uni, st);
        }
        return fail("the two-cell kernels need a float arithmetic type");
    }
    switch (storage) {
        case kF32: return launch_tick_t<float, false>(les, a, blocks, j, uni, st);
        case kF64: return launch_tick_t<double, false>(les, a, blocks, j, uni, st);
        case kF16: return launch_tick_t<__half, false>(les, a, blocks, j, uni, st);
        case kBF16: return launch_tick_t<__nv_bfloat16, false>(les, a, blocks, j, uni, st);
        case kC16: return launch_tick_t<c16_t, false>(les, a, blocks, j, uni, st);
    }
    return fail("unknown storage type");
}

// Bytes a cavity holds on the device (populations, flags, optional u).
size_t cavity_bytes(const lbm_cavity &c, int store_v) {
    const int64_t n = (int64_t)c.nx * c.ny * c.nz;
    const int64_t ps = round_up(n, 256 / (int64_t)storage_bytes(c.storage));
    return (size_t)ps * 19 * storage_bytes(c.storage) + (size_t)round_up(n, 256) +
           (store_v ? (size_t)n * 3 * real_bytes(c.storage) : 0) + 4096;
}

int check_cavity(const lbm_cavity &c) {
    if (c.nx < 3 || c.ny < 3 || c.nz < 3) return fail("cavity edges must be at least 3 cells");
    if (c.storage < LBM_F32 || c.storage > LBM_C16) return fail("unknown storage type");
    if (!(c.tau0 > 0.5)) return fail("cavity tau0 must exceed 0.5");
    if (c.steps < 0) return fail("negative step count");
    return 0;
}

// The kernel arguments of a cavity: inv_tau = 1/tau0 in its arithmetic type.
lbm_params cavity_params(const lbm_cavity &c) {
    lbm_params p{};
    if (c.storage == LBM_F64) {
        p.inv_tau = 1.0 / c.tau0;
        p.tau0 = c.tau0;
    } else {
        const float t = (float)c.tau0;
        p.inv_tau = (double)(1.0f / t);
        p.tau0 = (double)t;
    }
    p.les_c = 18.0 * std::sqrt(2.0) * c.cs * c.cs;
    p.lid = c.lid;
    return p;
}

// A lid-driven cavity at step 0: walls on all faces, the lid plane of
// CController::setGeometry (src/CController.hpp:531-546), optional seeded
// start-up.
int cavity_reset(lbm_lattice *l, const lbm_cavity &c, cudaStream_t st) {
    const int bc[6] = {LBM_FLAG_OBSTACLE, LBM_FLAG_OBSTACLE, LBM_FLAG_OBSTACLE,
                       LBM_FLAG_OBSTACLE, LBM_FLAG_OBSTACLE, LBM_FLAG_OBSTACLE};
    if (lbm_cu_init(l, bc, st)) return -1;
    const int o[3] = {1, c.ny - 2, 1}, sz[3] = {c.nx - 2, 1, c.nz - 2};
    std::vector<int32_t> lid((size_t)sz[0] * sz[2], LBM_FLAG_VELOCITY_INJECTION);
    if (lbm_cu_write(l, LBM_FIELD_FLAGS, o, sz, lid.data(), nullptr, st)) return -1;
    if (c.amp != 0.0) {
        const int zero[3] = {0, 0, 0}, phys[3] = {c.nx, c.ny, c.nz};
        if (lbm_cu_perturb(l, zero, phys, c.seed, c.amp, st)) return -1;
    }
    return 0;
}

struct Ensemble {
    struct Slot {
        lbm_cavity spec{};
        lbm_lattice *lat = nullptr;
        int64_t done = 0;
        bool active = false;
        int64_t id = -1;
    };
    // One launch per chunk of up to kBatchLattices members per step.
    struct Chunk {
        std::unique_ptr<BatchArgs> args;  // descriptors with this tick's parities
        std::unique_ptr<BatchArgs> sargs;  // the same numbered in staged tiles (staged groups)
        int blocks = 0;
        int tiles = 0;
        int parities = 0;  // bit p: some member's step counter has parity p
        bool les = false;
    };
    struct Group {
        int storage = 0;
        bool pair = false;
        bool staged = false;  // alpha steps through the staged tiles (shape 3, 16-bit storage)
        bool aligned = false;  // staged, and every nx a multiple of 16 bytes: beta steps staged too
        std::vector<int> members;
        std::vector<Chunk> chunks;
        int32_t *dmap = nullptr;  // lattice index (within its chunk) of every block
    };
    std::vector<Slot> slots;
    std::vector<Group> groups;
    int store_v = 0;
    int shape = 1;
    bool dirty = true;
    cudaGraphExec_t graph = nullptr;
    std::vector<int> graph_parity;  // parities baked into the captured graph
    cudaStream_t cap = nullptr;

    ~Ensemble() {
        drop_graph();
        if (cap) cudaStreamDestroy(cap);
        free_groups();
        for (auto &s : slots)
            if (s.lat) lbm_cu_destroy(s.lat);
    }
    void drop_graph() {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
    }
    void free_groups() {
        for (auto &g : groups)
            if (g.dmap) cudaFree(g.dmap);
        groups.clear();
    }

    // Member groups of the active cavities, one per (storage, shape), and
    // their block maps.
    int build_groups() {
        free_groups();
        for (size_t i = 0; i < slots.size(); i++) {
            const Slot &s = slots[i];
            if (!s.active) continue;
            const bool pair = shape == 2 && s.spec.storage != LBM_F64 && !(s.spec.nx & 1);
            const bool staged =
                shape == 3 && (s.spec.storage == LBM_F16 || s.spec.storage == LBM_BF16 || s.spec.storage == LBM_C16);
            const bool aligned = staged && ((int64_t)s.spec.nx * storage_bytes(s.spec.storage)) % 16 == 0;
            Group *g = nullptr;
            for (auto &x : groups)
                if (x.storage == s.spec.storage && x.pair == pair && x.aligned == aligned) g = &x;
            if (!g) {
                groups.emplace_back();
                g = &groups.back();
                g->storage = s.spec.storage;
                g->pair = pair;
                g->staged = staged;
                g->aligned = aligned;
            }
            g->members.push_back((int)i);
        }
        for (auto &g : groups) {
            const int per = cells_per_block(g.pair);
            std::vector<int32_t> map;
            for (size_t k = 0; k < g.members.size(); k++) {
                const int64_t n = slots[g.members[k]].lat->n;
                map.insert(map.end(), (size_t)((n + per - 1) / per), (int32_t)(k % kBatchLattices));
            }
            CU(cudaMalloc((void **)&g.dmap, map.size() * sizeof(int32_t)));
            CU(cudaMemcpy(g.dmap, map.data(), map.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
            g.chunks.resize((g.members.size() + kBatchLattices - 1) / kBatchLattices);
            for (auto &c : g.chunks) {
                c.args.reset(new BatchArgs());
                if (g.staged) c.sargs.reset(new BatchArgs());
            }
        }
        dirty = false;
        drop_graph();
        return refresh_tables();
    }

    // Descriptors with the current step-counter parities (and block
    // numbering) into the launch arguments; a graph captured with other
    // parities is dropped.
    int refresh_tables() {
        std::vector<int> parity;
        for (auto &g : groups) {
            const int per = cells_per_block(g.pair);
            int64_t map_off = 0;
            for (size_t c = 0; c < g.chunks.size(); c++) {
                Chunk &ch = g.chunks[c];
                BatchArgs &a = *ch.args;
                memset(&a, 0, sizeof(a));
                const size_t k0 = c * kBatchLattices, k1 = std::min(g.members.size(), k0 + kBatchLattices);
                int first = 0, tile = 0;
                const int tcells = g.staged ? staged_cells(g.storage) : 0;
                if (g.staged) memset(ch.sargs.get(), 0, sizeof(BatchArgs));
                ch.les = false;
                ch.parities = 0;
                for (size_t k = k0; k < k1; k++) {
                    const Slot &s = slots[g.members[k]];
                    LatDesc h = s.lat->h;
                    h.first_block = first;
                    h.nblocks = (int)((h.n + per - 1) / per);
                    h.parity = (int)(s.done & 1);
                    first += h.nblocks;
                    if (uses_les(h)) ch.les = true;
                    a.tab[k - k0] = h;
                    parity.push_back(h.parity);
                    ch.parities |= 1 << h.parity;
                    if (g.staged) {
                        h.first_block = tile;
                        h.nblocks = (int)((h.n + tcells - 1) / tcells);
                        tile += h.nblocks;
                        ch.sargs->tab[k - k0] = h;
                    }
                }
                a.ntab = (int)(k1 - k0);
                a.block_lattice = g.dmap + map_off;
                ch.blocks = first;
                map_off += first;
                if (g.staged) ch.sargs->ntab = a.ntab;
                ch.tiles = tile;
            }
        }
        if (parity != graph_parity) drop_graph();
        graph_parity = parity;
        return 0;
    }

    int launch_all(int j, bool store, cudaStream_t st) {
        for (auto &g : groups)
            for (auto &ch : g.chunks) {
                const bool all_alpha = ch.parities == 1 << ((j + 1) & 1);
                const bool all_beta = ch.parities == 1 << (j & 1);
                if (g.staged && (all_alpha || (all_beta && g.aligned))) {
                    // every member at the same kind of step: staged tiles
                    ch.sargs->store_v = store ? store_v : 0;
                    ch.sargs->store_rho = 0;
                    if (launch_staged_batch(g.storage, all_beta, ch.les, *ch.sargs, ch.tiles, st)) return -1;
                    continue;
                }
                ch.args->store_v = store ? store_v : 0;
                ch.args->store_rho = 0;
                if (launch_tick(g.storage, g.pair, ch.les, *ch.args, ch.blocks, j, all_alpha ? 1 : all_beta ? 2 : 0, st))
                    return -1;
            }
        return 0;
    }

    int64_t active_count() const {
        int64_t n = 0;
        for (auto &s : slots) n += s.active;
        return n;
    }

    // Advance every active cavity by k steps; the last step writes u.
    int tick(int64_t k, bool use_graph, cudaStream_t st) {
        if (k <= 0 || active_count() == 0) return 0;
        CU(cudaStreamSynchronize(st));
        if (dirty) {
            if (build_groups()) return -1;
        } else if (refresh_tables()) {
            return -1;
        }
        const int64_t plain = k - 1;
        int64_t j = 0;
        if (use_graph && plain >= 2) {
            if (!graph) {
                if (!cap) CU(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
                cudaGraph_t g = nullptr;
                CU(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
                int rc = launch_all(0, false, cap);
                if (!rc) rc = launch_all(1, false, cap);
                cudaError_t e = cudaStreamEndCapture(cap, &g);
                if (rc) {
                    if (g) cudaGraphDestroy(g);
                    return -1;
                }
                if (e != cudaSuccess) return fail(std::string("graph capture: ") + cudaGetErrorString(e));
                e = cudaGraphInstantiate(&graph, g, 0);
                cudaGraphDestroy(g);
                if (e != cudaSuccess) {
                    graph = nullptr;
                    return fail(std::string("graph instantiate: ") + cudaGetErrorString(e));
                }
            }
            const int64_t reps = plain / 2;
            for (int64_t r = 0; r < reps; r++) CU(cudaGraphLaunch(graph, st));
            j = 2 * reps;
        }
        for (; j < plain; j++)
            if (launch_all((int)(j & 1), false, st)) return -1;
        if (launch_all((int)((k - 1) & 1), true, st)) return -1;
        for (auto &s : slots)
            if (s.active) s.done += k;
        return 0;
    }

    // Steps until the first active cavity completes.
    int64_t min_remaining() const {
        int64_t m = INT64_MAX;
        for (auto &s : slots)
            if (s.active) m = std::min(m, s.spec.steps - s.done);
        return m == INT64_MAX ? 0 : m;
    }

    // Cavities that reached their step count stop taking steps.
    void retire_finished() {
        for (auto &s : slots)
            if (s.active && s.done >= s.spec.steps) {
                s.active = false;
                dirty = true;
            }
    }
};

}  // namespace lbm_rt

struct lbm_batch {
    Ensemble e;
};

struct lbm_server {
    Ensemble e;
    double budget = 0;  // bytes of HBM the resident solves may hold
    double used = 0;
    int max_active = 0;
    int64_t next_id = 0;
    struct Pending {
        int64_t id;
        lbm_cavity spec;
    };
    std::deque<Pending> queue;
    std::vector<int64_t> completed;  // finished since the last poll
    std::vector<int> free_slots;
    int64_t cell_updates = 0;
};

extern "C" {

// ---------------------------------------------------------------- one lattice
int lbm_cu_run(lbm_lattice *lat, int64_t first_step, int64_t steps, void *stream) {
    if (!lat) return fail("NULL lattice");
    for (int64_t t = 0; t < steps; t++)
        if (lbm_cu_step(lat, (int)((first_step + t) & 1), stream)) return -1;
    return 0;
}

// ------------------------------------------------------------------- batch
int lbm_cu_batch_create(const lbm_cavity *cav, int count, int store_velocity, lbm_batch **out) {
    if (!cav || !out || count < 0) return fail("bad argument");
    *out = nullptr;
    lbm_batch *b = new lbm_batch();
    b->e.store_v = store_velocity ? 1 : 0;
    for (int i = 0; i < count; i++) {
        if (check_cavity(cav[i])) {
            std::string m = "cavity " + std::to_string(i) + ": " + lbm_cu_last_error();
            delete b;
            return fail(m);
        }
        Ensemble::Slot s;
        s.spec = cav[i];
        s.id = i;
        if (lbm_cu_create(cav[i].nx, cav[i].ny, cav[i].nz, cav[i].storage, b->e.store_v, 0, &s.lat)) {
            std::string m = "cavity " + std::to_string(i) + ": " + lbm_cu_last_error();
            delete b;
            return fail(m);
        }
        const lbm_params p = cavity_params(cav[i]);
        if (lbm_cu_set_params(s.lat, &p)) {
            std::string m = lbm_cu_last_error();
            lbm_cu_destroy(s.lat);
            delete b;
            return fail(m);
        }
        b->e.slots.push_back(s);
    }
    *out = b;
    return 0;
}

int lbm_cu_batch_destroy(lbm_batch *b) {
    delete b;
    return 0;
}

int lbm_cu_batch_reset(lbm_batch *b, void *stream) {
    if (!b) return fail("NULL batch");
    for (auto &s : b->e.slots) {
        if (cavity_reset(s.lat, s.spec, S(stream))) return -1;
        s.done = 0;
        s.active = s.spec.steps > 0;
    }
    b->e.dirty = true;
    return 0;
}

int lbm_cu_batch_set_kernel_shape(lbm_batch *b, int cells_per_thread) {
    if (!b) return fail("NULL batch");
    if (cells_per_thread < 1 || cells_per_thread > 3) return fail("the ensemble kernel shape is 1, 2 or 3");
    b->e.shape = cells_per_thread;
    b->e.dirty = true;
    return 0;
}

int lbm_cu_batch_run(lbm_batch *b, int64_t max_steps, int use_graph, void *stream) {
    if (!b) return fail("NULL batch");
    int64_t budget = max_steps < 0 ? INT64_MAX : max_steps;
    b->e.retire_finished();
    while (budget > 0 && b->e.active_count() > 0) {
        const int64_t k = std::min(budget, b->e.min_remaining());
        if (b->e.tick(k, use_graph != 0, S(stream))) return -1;
        budget -= k;
        b->e.retire_finished();
    }
    CU(cudaStreamSynchronize(S(stream)));
    return 0;
}

int lbm_cu_batch_tune(lbm_batch *b, int trial_steps, int *cells_per_thread, double *ms_per_step, void *stream) {
    if (!b || trial_steps < 1) return fail("bad argument");
    cudaStream_t st = S(stream);
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    double best_ms = 1e300;
    int best = 1;
    for (int shape = 1; shape <= 3; shape++) {
        b->e.shape = shape;
        b->e.dirty = true;
        if (lbm_cu_batch_reset(b, stream)) return -1;
        if (b->e.tick(2, true, st)) return -1;  // warm-up (and table build)
        CU(cudaEventRecord(e0, st));
        if (b->e.tick(trial_steps, true, st)) return -1;
        CU(cudaEventRecord(e1, st));
        CU(cudaEventSynchronize(e1));
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
            best_ms = ms;
            best = shape;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->e.shape = best;
    b->e.dirty = true;
    if (lbm_cu_batch_reset(b, stream)) return -1;
    if (cells_per_thread) *cells_per_thread = best;
    if (ms_per_step) *ms_per_step = best_ms / trial_steps;
    return 0;
}

int lbm_cu_batch_status(const lbm_batch *b, int64_t *min_done, int *active) {
    if (!b) return fail("NULL batch");
    int64_t m = INT64_MAX;
    int a = 0;
    for (auto &s : b->e.slots) {
        m = std::min(m, s.done);
        a += s.active;
    }
    if (min_done) *min_done = m == INT64_MAX ? 0 : m;
    if (active) *active = a;
    return 0;
}

lbm_lattice *lbm_cu_batch_lattice(lbm_batch *b, int index) {
    if (!b || index < 0 || index >= (int)b->e.slots.size()) {
        fail("cavity index out of range");
        return nullptr;
    }
    return b->e.slots[index].lat;
}

// ------------------------------------------------------------------ server
int lbm_cu_server_create(double hbm_budget_bytes, int max_active, int store_velocity, lbm_server **out) {
    if (!out || !(hbm_budget_bytes > 0)) return fail("bad argument");
    lbm_server *s = new lbm_server();
    s->budget = hbm_budget_bytes;
    s->max_active = max_active > 0 ? max_active : 1 << 30;
    s->e.store_v = store_velocity ? 1 : 0;
    s->e.shape = 3;  // staged alpha steps for parity-uniform 16-bit launches (measured the faster)
    *out = s;
    return 0;
}

int lbm_cu_server_destroy(lbm_server *s) {
    delete s;
    return 0;
}

int lbm_cu_server_set_kernel_shape(lbm_server *s, int cells_per_thread) {
    if (!s) return fail("NULL server");
    if (cells_per_thread < 1 || cells_per_thread > 3) return fail("the ensemble kernel shape is 1, 2 or 3");
    s->e.shape = cells_per_thread;
    s->e.dirty = true;
    return 0;
}

int lbm_cu_server_submit(lbm_server *s, const lbm_cavity *c, int64_t *id) {
    if (!s || !c) return fail("NULL argument");
    if (check_cavity(*c)) return -1;
    if (cavity_bytes(*c, s->e.store_v) > s->budget) return fail("solve does not fit the HBM budget");
    lbm_server::Pending p{s->next_id++, *c};
    s->queue.push_back(p);
    if (id) *id = p.id;
    return 0;
}

// Admit queued solves in arrival order while the budget and slot limit
// allow; returns the number admitted.
static int server_admit(lbm_server *s, cudaStream_t st) {
    int admitted = 0;
    while (!s->queue.empty()) {
        const lbm_server::Pending &p = s->queue.front();
        const double need = (double)cavity_bytes(p.spec, s->e.store_v);
        if (s->used + need > s->budget || s->e.active_count() >= s->max_active) break;
        Ensemble::Slot slot;
        slot.spec = p.spec;
        slot.id = p.id;
        if (lbm_cu_create(p.spec.nx, p.spec.ny, p.spec.nz, p.spec.storage, s->e.store_v, 0, &slot.lat)) return -1;
        const lbm_params prm = cavity_params(p.spec);
        if (lbm_cu_set_params(slot.lat, &prm) || cavity_reset(slot.lat, p.spec, st)) {
            lbm_cu_destroy(slot.lat);
            return -1;
        }
        slot.active = p.spec.steps > 0;
        if (!slot.active) s->completed.push_back(p.id);  // nothing to run
        if (!s->free_slots.empty()) {
            s->e.slots[s->free_slots.back()] = slot;
            s->free_slots.pop_back();
        } else {
            s->e.slots.push_back(slot);
        }
        s->used += need;
        s->queue.pop_front();
        s->e.dirty = true;
        admitted++;
    }
    return admitted;
}

int lbm_cu_server_tick(lbm_server *s, int64_t max_steps, int use_graph, int *admitted, void *stream) {
    if (!s) return fail("NULL server");
    cudaStream_t st = S(stream);
    const int adm = server_admit(s, st);
    if (adm < 0) return -1;
    if (admitted) *admitted = adm;
    const int64_t k = std::min(max_steps > 0 ? max_steps : INT64_MAX, s->e.min_remaining());
    if (k > 0) {
        int64_t cells = 0;
        for (auto &sl : s->e.slots)
            if (sl.active) cells += sl.lat->n;
        if (s->e.tick(k, use_graph != 0, st)) return -1;
        s->cell_updates += cells * k;
    }
    for (auto &sl : s->e.slots)
        if (sl.active && sl.done >= sl.spec.steps) {
            sl.active = false;
            s->e.dirty = true;
            s->completed.push_back(sl.id);
        }
    CU(cudaStreamSynchronize(st));
    return 0;
}

int lbm_cu_server_poll(lbm_server *s, int64_t *ids, int capacity, int *count) {
    if (!s || !count) return fail("NULL argument");
    const int n = std::min<int>(capacity, (int)s->completed.size());
    for (int i = 0; i < n; i++) ids[i] = s->completed[i];
    s->completed.erase(s->completed.begin(), s->completed.begin() + n);
    *count = n;
    return 0;
}

// The lattice of a completed (or running) solve, for readback.
lbm_lattice *lbm_cu_server_lattice(lbm_server *s, int64_t id) {
    if (!s) return nullptr;
    for (auto &sl : s->e.slots)
        if (sl.lat && sl.id == id) return sl.lat;
    fail("no resident solve with this id");
    return nullptr;
}

// Free a completed solve's device memory and return its slot.
int lbm_cu_server_release(lbm_server *s, int64_t id) {
    if (!s) return fail("NULL server");
    for (size_t i = 0; i < s->e.slots.size(); i++) {
        auto &sl = s->e.slots[i];
        if (sl.lat && sl.id == id) {
            if (sl.active) return fail("solve is still running");
            s->used -= (double)cavity_bytes(sl.spec, s->e.store_v);
            lbm_cu_destroy(sl.lat);
            sl = Ensemble::Slot();
            s->free_slots.push_back((int)i);
            return 0;
        }
    }
    return fail("no resident solve with this id");
}

int lbm_cu_server_status(const lbm_server *s, int *queued, int *active, double *hbm_used, int64_t *cell_updates) {
    if (!s) return fail("NULL server");
    if (queued) *queued = (int)s->queue.size();
    if (active) *active = (int)s->e.active_count();
    if (hbm_used) *hbm_used = s->used;
    if (cell_updates) *cell_updates = s->cell_updates;
    return 0;
}

}  // extern "C"
