/*
 * fsm_oracle.c -- CPU oracle for the automata-simulation hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle that the CUDA path is compared
 * against; it is never linked into, loaded by or called from the product library or
 * its Python package. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg load it (through oracle/oracle.py).
 *
 * It restates, in plain C, the latch-first-match simulators of the reference package
 * gpufsm 0.1.0 (alepot55/abstraction-regret):
 *
 *   nfa_one()      <- src/gpufsm/reference.py:36-65   simulate()
 *   closure()      <- src/gpufsm/reference.py:20-33   epsilon_closure() (iterative DFS)
 *   dfa_one()      <- src/gpufsm/reference.py:68-81   simulate_dfa()
 *
 * Semantics kept exactly (the reference's order of tests):
 *   - the start configuration is the epsilon closure of {start}; if any state of it
 *     accepts, the verdict is (1, 0) and no byte is consumed;
 *   - for byte i: next = { target(e) : e an edge of an active state, sym(e) == byte or
 *     sym(e) == ANY (256) }; an empty next set ends the run with (0, 0)
 *     (reference.py:59-60); otherwise next is closed under epsilon edges and, if any
 *     state of it accepts, the verdict is (1, i + 1);
 *   - running off the end of the input gives (0, 0).
 *   DFA: cur = start; accept[start] gives (1, 0); then cur = trans[cur * 256 + byte] and
 *   the first accepting cur gives (1, i + 1); otherwise (0, 0).
 *
 * Two outputs that the reference does not compute are added for measurement only:
 *   examined[i]   bytes consumed before the run ended (latch position, the byte on which
 *                 the set died, or the whole input);
 *   max_active[i] the largest active-set size seen (start closure included), which is
 *                 what a "divergence > 1" input filter looks at;
 *   work[i]       symbol edges scanned over the run (the sum over consumed bytes of the
 *                 out-degrees of the active states), which sizes a simulator's edge
 *                 traffic per byte;
 *   visits[i]     active states stepped over the run (the sum over consumed bytes of the
 *                 active-set size), which sizes its row-pointer traffic.
 *
 * Sets are a membership byte map plus a member list (O(1) insert, O(|set|) iteration
 * and clear), so a run costs O(edges touched), like the reference's Python sets.
 * Batches are spread over POSIX threads; each thread owns its scratch.
 *
 * Parity of this file is pinned by tests/test_oracle.py against the reference's own
 * golden corpus (tests/data/golden.json of the reference, re-serialised under
 * tests/golden/) and against golden vectors generated by importing the reference.
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_ANY_SYMBOL 256
#define ORACLE_ALPHABET 256

typedef struct {
    int32_t n, start;
    const uint8_t *accept;
    const int32_t *srp, *stg, *ssy, *erp, *etg;
} nfa_t;

typedef struct {
    uint8_t *in_cur, *in_nxt; /* membership maps, n bytes each */
    int32_t *cur, *nxt;       /* member lists, n entries each */
    int32_t *stack;           /* DFS stack, n entries */
} scratch_t;

/* Close the set {list[0..*count)} (membership in `in`) under epsilon edges with an
 * iterative depth-first search, as reference.py:20-33 does. Returns 1 if any member
 * accepts. */
static int closure(const nfa_t *a, int32_t *list, int32_t *count, uint8_t *in, int32_t *stack) {
    int32_t top = 0;
    for (int32_t j = 0; j < *count; ++j) stack[top++] = list[j];
    while (top > 0) {
        int32_t s = stack[--top];
        for (int32_t k = a->erp[s]; k < a->erp[s + 1]; ++k) {
            int32_t t = a->etg[k];
            if (!in[t]) {
                in[t] = 1;
                list[(*count)++] = t;
                stack[top++] = t;
            }
        }
    }
    int acc = 0;
    for (int32_t j = 0; j < *count; ++j) acc |= a->accept[list[j]] != 0;
    return acc;
}

static void nfa_one(const nfa_t *a, scratch_t *w, const uint8_t *data, int64_t len,
                    int32_t *flag, int32_t *mlen, int64_t *examined, int32_t *max_active,
                    int64_t *work, int64_t *visits) {
    int64_t edges = 0, stepped = 0;
    int32_t nc = 0, nn = 0, peak;
    w->cur[nc++] = a->start;
    w->in_cur[a->start] = 1;
    int acc = closure(a, w->cur, &nc, w->in_cur, w->stack);
    peak = nc;
    int32_t f = 0, l = 0;
    int64_t ex = 0;
    if (acc) {
        f = 1;
    } else {
        int64_t i;
        for (i = 0; i < len; ++i) {
            int32_t b = data[i];
            nn = 0;
            stepped += nc;
            for (int32_t j = 0; j < nc; ++j) {
                int32_t s = w->cur[j];
                edges += a->srp[s + 1] - a->srp[s];
                for (int32_t k = a->srp[s]; k < a->srp[s + 1]; ++k) {
                    int32_t sym = a->ssy[k];
                    if (sym == b || sym == ORACLE_ANY_SYMBOL) {
                        int32_t t = a->stg[k];
                        if (!w->in_nxt[t]) {
                            w->in_nxt[t] = 1;
                            w->nxt[nn++] = t;
                        }
                    }
                }
            }
            /* the current set is replaced: clear its membership map in O(|set|) */
            for (int32_t j = 0; j < nc; ++j) w->in_cur[w->cur[j]] = 0;
            if (nn == 0) { /* reference.py:59-60: an empty set ends the run */
                nc = 0;
                ex = i + 1;
                break;
            }
            acc = closure(a, w->nxt, &nn, w->in_nxt, w->stack);
            /* swap cur <-> nxt */
            int32_t *tl = w->cur; w->cur = w->nxt; w->nxt = tl;
            uint8_t *tm = w->in_cur; w->in_cur = w->in_nxt; w->in_nxt = tm;
            nc = nn;
            if (nc > peak) peak = nc;
            if (acc) {
                f = 1;
                l = (int32_t)(i + 1);
                ex = i + 1;
                break;
            }
        }
        if (i == len) ex = len;
    }
    for (int32_t j = 0; j < nc; ++j) w->in_cur[w->cur[j]] = 0;
    *flag = f;
    *mlen = l;
    if (examined) *examined = ex;
    if (max_active) *max_active = peak;
    if (work) *work = edges;
    if (visits) *visits = stepped;
}

/* Reject automata the simulator would index out of bounds with. Returns 0 when valid. */
static int nfa_valid(const nfa_t *a) {
    if (a->n < 1 || a->start < 0 || a->start >= a->n) return -1;
    if (a->srp[0] != 0 || a->erp[0] != 0) return -1;
    for (int32_t s = 0; s < a->n; ++s)
        if (a->srp[s + 1] < a->srp[s] || a->erp[s + 1] < a->erp[s]) return -1;
    for (int32_t k = 0; k < a->srp[a->n]; ++k) {
        if (a->stg[k] < 0 || a->stg[k] >= a->n) return -1;
        if (a->ssy[k] < 0 || a->ssy[k] > ORACLE_ANY_SYMBOL) return -1;
    }
    for (int32_t k = 0; k < a->erp[a->n]; ++k)
        if (a->etg[k] < 0 || a->etg[k] >= a->n) return -1;
    return 0;
}

typedef struct {
    const nfa_t *nfa;
    int32_t dfa_n, dfa_start;
    const uint8_t *dfa_accept;
    const int32_t *dfa_trans;
    const uint8_t *data;
    const int64_t *offsets;
    int64_t n_inputs;
    int64_t next; /* shared work counter */
    int32_t *flags, *lens, *max_active;
    int64_t *examined, *work, *visits;
    int failed;
} job_t;

static void *nfa_worker(void *arg) {
    job_t *job = (job_t *)arg;
    const nfa_t *a = job->nfa;
    scratch_t w;
    w.in_cur = (uint8_t *)calloc((size_t)a->n, 1);
    w.in_nxt = (uint8_t *)calloc((size_t)a->n, 1);
    w.cur = (int32_t *)malloc(sizeof(int32_t) * (size_t)a->n);
    w.nxt = (int32_t *)malloc(sizeof(int32_t) * (size_t)a->n);
    w.stack = (int32_t *)malloc(sizeof(int32_t) * (size_t)a->n);
    if (!w.in_cur || !w.in_nxt || !w.cur || !w.nxt || !w.stack) {
        __atomic_store_n(&job->failed, 1, __ATOMIC_RELAXED);
    } else {
        for (;;) {
            int64_t i = __atomic_fetch_add(&job->next, 1, __ATOMIC_RELAXED);
            if (i >= job->n_inputs) break;
            nfa_one(a, &w, job->data + job->offsets[i], job->offsets[i + 1] - job->offsets[i],
                    &job->flags[i], &job->lens[i], job->examined ? &job->examined[i] : NULL,
                    job->max_active ? &job->max_active[i] : NULL,
                    job->work ? &job->work[i] : NULL,
                    job->visits ? &job->visits[i] : NULL);
        }
    }
    free(w.in_cur); free(w.in_nxt); free(w.cur); free(w.nxt); free(w.stack);
    return NULL;
}

static void dfa_one(const job_t *job, const uint8_t *data, int64_t len,
                    int32_t *flag, int32_t *mlen, int64_t *examined) {
    int32_t cur = job->dfa_start;
    int32_t f = 0, l = 0;
    int64_t ex = len;
    if (job->dfa_accept[cur]) {
        f = 1;
        ex = 0;
    } else {
        for (int64_t i = 0; i < len; ++i) {
            cur = job->dfa_trans[(int64_t)cur * ORACLE_ALPHABET + data[i]];
            if (job->dfa_accept[cur]) {
                f = 1;
                l = (int32_t)(i + 1);
                ex = i + 1;
                break;
            }
        }
    }
    *flag = f;
    *mlen = l;
    if (examined) *examined = ex;
}

static void *dfa_worker(void *arg) {
    job_t *job = (job_t *)arg;
    for (;;) {
        int64_t i = __atomic_fetch_add(&job->next, 1, __ATOMIC_RELAXED);
        if (i >= job->n_inputs) break;
        dfa_one(job, job->data + job->offsets[i], job->offsets[i + 1] - job->offsets[i],
                &job->flags[i], &job->lens[i], job->examined ? &job->examined[i] : NULL);
    }
    return NULL;
}

static int run_pool(job_t *job, int32_t n_threads, void *(*fn)(void *)) {
    if (n_threads < 1) n_threads = 1;
    if (n_threads > 256) n_threads = 256;
    if ((int64_t)n_threads > job->n_inputs) n_threads = (int32_t)(job->n_inputs > 0 ? job->n_inputs : 1);
    pthread_t tids[256];
    int32_t started = 0;
    for (int32_t t = 1; t < n_threads; ++t) {
        if (pthread_create(&tids[started], NULL, fn, job) != 0) break;
        ++started;
    }
    fn(job); /* the calling thread works too */
    for (int32_t t = 0; t < started; ++t) pthread_join(tids[t], NULL);
    return job->failed ? -2 : 0;
}

static int offsets_valid(const int64_t *offsets, int64_t n_inputs) {
    if (n_inputs < 0) return -1;
    if (offsets[0] < 0) return -1;
    for (int64_t i = 0; i < n_inputs; ++i)
        if (offsets[i + 1] < offsets[i]) return -1;
    return 0;
}

/* NFA batch: input i is data[offsets[i] .. offsets[i+1]). `examined`, `max_active` and
 * `work` may be NULL. Returns 0, -1 for an invalid automaton or offsets, -2 on allocation
 * failure. */
int fsm_oracle_nfa_batch(int32_t num_states, int32_t start_state, const uint8_t *accept,
                         const int32_t *sym_row_ptr, const int32_t *sym_targets,
                         const int32_t *sym_symbols, const int32_t *eps_row_ptr,
                         const int32_t *eps_targets, const uint8_t *data,
                         const int64_t *offsets, int64_t n_inputs, int32_t n_threads,
                         int32_t *flags, int32_t *lens, int64_t *examined,
                         int32_t *max_active, int64_t *work, int64_t *visits) {
    nfa_t a = {num_states, start_state, accept, sym_row_ptr, sym_targets, sym_symbols,
               eps_row_ptr, eps_targets};
    if (nfa_valid(&a) != 0 || offsets_valid(offsets, n_inputs) != 0) return -1;
    job_t job;
    memset(&job, 0, sizeof(job));
    job.nfa = &a;
    job.data = data;
    job.offsets = offsets;
    job.n_inputs = n_inputs;
    job.flags = flags;
    job.lens = lens;
    job.examined = examined;
    job.max_active = max_active;
    job.work = work;
    job.visits = visits;
    return run_pool(&job, n_threads, nfa_worker);
}

/* DFA batch over a dense table trans[num_states * 256]. Returns 0 or -1 (invalid). */
int fsm_oracle_dfa_batch(int32_t num_states, int32_t start_state, const uint8_t *accept,
                         const int32_t *trans, const uint8_t *data, const int64_t *offsets,
                         int64_t n_inputs, int32_t n_threads, int32_t *flags, int32_t *lens,
                         int64_t *examined) {
    if (num_states < 1 || start_state < 0 || start_state >= num_states) return -1;
    for (int64_t k = 0; k < (int64_t)num_states * ORACLE_ALPHABET; ++k)
        if (trans[k] < 0 || trans[k] >= num_states) return -1;
    if (offsets_valid(offsets, n_inputs) != 0) return -1;
    job_t job;
    memset(&job, 0, sizeof(job));
    job.dfa_n = num_states;
    job.dfa_start = start_state;
    job.dfa_accept = accept;
    job.dfa_trans = trans;
    job.data = data;
    job.offsets = offsets;
    job.n_inputs = n_inputs;
    job.flags = flags;
    job.lens = lens;
    job.examined = examined;
    return run_pool(&job, n_threads, dfa_worker);
}

/* ---- random-walk input generator for the CPU reference arm ------------------------------
 *
 * The benchmark's "live" and "sustained" inputs are random walks through an automaton's
 * live core; the product library generates them for the GPU arm. The CPU reference arm
 * must not load the product library, so it generates the same bytes here. The walk:
 *   - live core = the largest set of non-accepting states in which every state has a
 *     symbol edge to another state of the set (prune states without such an edge until
 *     nothing changes);
 *   - input i uses a SplitMix64 stream (Steele, Lea & Flood, OOPSLA 2014) seeded with
 *     seed * 0x100000001b3 ^ (i + 1) * 0x9e3779b97f4a7c15; at each position the walk
 *     state draws one of its edges into the core uniformly (multiply-shift of the top 32
 *     bits), emits the edge's symbol (a draw's low byte for ANY) and moves on;
 *   - once the walk is outside the core (or the core gives no edge), the rest of the
 *     input is the low bytes of successive draws.
 * tests/test_oracle.py checks that both generators give identical bytes. */

typedef struct {
    uint64_t s;
} mix_t;

static uint64_t mix_next(mix_t *r) {
    uint64_t z = (r->s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

static uint32_t mix_below(mix_t *r, uint32_t n) {
    return (uint32_t)(((mix_next(r) >> 32) * (uint64_t)n) >> 32);
}

/* live[s] = 1 for the states of the live core; returns -2 on allocation failure. */
static int live_states(int32_t n, const int32_t *srp, const int32_t *stg, const uint8_t *accept,
                       uint8_t *live) {
    const int32_t nnz = srp[n];
    int32_t *deg = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    int32_t *rrow = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
    int32_t *pos = (int32_t *)malloc(sizeof(int32_t) * ((size_t)n + 1));
    int32_t *rsrc = (int32_t *)malloc(sizeof(int32_t) * ((size_t)nnz + 1));
    int32_t *queue = (int32_t *)malloc(sizeof(int32_t) * ((size_t)n + 1));
    int rc = 0;
    if (!deg || !rrow || !pos || !rsrc || !queue) {
        rc = -2;
        goto out;
    }
    /* reverse edges, and each state's count of edges into non-accepting states */
    for (int32_t k = 0; k < nnz; ++k)
        if (stg[k] >= 0 && stg[k] < n) rrow[stg[k] + 1]++;
    for (int32_t s = 0; s < n; ++s) rrow[s + 1] += rrow[s];
    memcpy(pos, rrow, sizeof(int32_t) * (size_t)n);
    for (int32_t s = 0; s < n; ++s) {
        for (int32_t k = srp[s]; k < srp[s + 1]; ++k) {
            const int32_t t = stg[k];
            if (t < 0 || t >= n) continue;
            rsrc[pos[t]++] = s;
            if (!accept[t]) deg[s]++;
        }
    }
    int32_t qn = 0;
    for (int32_t s = 0; s < n; ++s) {
        live[s] = (uint8_t)!(accept[s] || deg[s] == 0);
        if (!live[s]) queue[qn++] = s;
    }
    for (int32_t q = 0; q < qn; ++q) {
        const int32_t t = queue[q];
        if (accept[t]) continue; /* its in-edges were never counted */
        for (int32_t r = rrow[t]; r < rrow[t + 1]; ++r) {
            const int32_t s = rsrc[r];
            if (live[s] && --deg[s] == 0) {
                live[s] = 0;
                queue[qn++] = s;
            }
        }
    }
out:
    free(deg);
    free(rrow);
    free(pos);
    free(rsrc);
    free(queue);
    return rc;
}

typedef struct {
    int32_t n, start;
    const int32_t *srp, *stg, *ssy;
    const uint8_t *live;
    const int64_t *offsets;
    int64_t n_inputs;
    uint64_t seed;
    uint8_t *out;
    int32_t stride;
    int32_t next_worker;
    int32_t max_degree;
    int32_t failed;
    pthread_mutex_t mu;
} walk_job_t;

static void walk_one_input(const walk_job_t *job, int64_t i, int32_t *good) {
    mix_t r = {job->seed * 0x100000001b3ull ^ (uint64_t)(i + 1) * 0x9e3779b97f4a7c15ull};
    uint8_t *o = job->out + job->offsets[i];
    const int64_t len = job->offsets[i + 1] - job->offsets[i];
    int32_t s = job->start;
    int64_t p = 0;
    for (; p < len && job->live[s]; ++p) {
        int32_t ng = 0;
        for (int32_t k = job->srp[s]; k < job->srp[s + 1]; ++k) {
            const int32_t t = job->stg[k];
            if (t >= 0 && t < job->n && job->live[t]) good[ng++] = k;
        }
        if (ng == 0) break;
        const int32_t k = good[mix_below(&r, (uint32_t)ng)];
        const int32_t sym = job->ssy[k];
        o[p] = (sym >= 0 && sym <= 255) ? (uint8_t)sym : (uint8_t)(mix_next(&r) & 0xffu);
        s = job->stg[k];
    }
    for (; p < len; ++p) o[p] = (uint8_t)(mix_next(&r) & 0xffu);
}

/* Each call claims stripes (inputs me, me + stride, ...) until none is left, so every
 * stripe is generated once whether or not all threads could be started. */
static void *walk_worker(void *arg) {
    walk_job_t *job = (walk_job_t *)arg;
    int32_t *good = (int32_t *)malloc(sizeof(int32_t) * ((size_t)job->max_degree + 1));
    for (;;) {
        pthread_mutex_lock(&job->mu);
        const int32_t me = job->next_worker++;
        if (!good) job->failed = 1;
        pthread_mutex_unlock(&job->mu);
        if (me >= job->stride || !good) break;
        for (int64_t i = me; i < job->n_inputs; i += job->stride) walk_one_input(job, i, good);
    }
    free(good);
    return NULL;
}

/* Random-walk inputs: out[offsets[i] .. offsets[i+1]) for every input i (see above).
 * Returns 0, -1 for invalid arguments, -2 on allocation failure. */
int fsm_oracle_walk(int32_t num_states, const int32_t *sym_row_ptr, const int32_t *sym_targets,
                    const int32_t *sym_symbols, const uint8_t *accept, int32_t start_state,
                    const int64_t *offsets, int64_t n_inputs, uint64_t seed, uint8_t *out,
                    int32_t n_threads) {
    if (num_states < 1 || start_state < 0 || start_state >= num_states || n_inputs < 0 ||
        !sym_row_ptr || !accept || !offsets || !out || offsets_valid(offsets, n_inputs) != 0)
        return -1;
    uint8_t *live = (uint8_t *)malloc((size_t)num_states);
    if (!live) return -2;
    int rc = live_states(num_states, sym_row_ptr, sym_targets, accept, live);
    if (rc != 0) {
        free(live);
        return rc;
    }
    walk_job_t job;
    memset(&job, 0, sizeof(job));
    job.n = num_states;
    job.start = start_state;
    job.srp = sym_row_ptr;
    job.stg = sym_targets;
    job.ssy = sym_symbols;
    job.live = live;
    job.offsets = offsets;
    job.n_inputs = n_inputs;
    job.seed = seed;
    job.out = out;
    for (int32_t s = 0; s < num_states; ++s) {
        const int32_t d = sym_row_ptr[s + 1] - sym_row_ptr[s];
        if (d > job.max_degree) job.max_degree = d;
    }
    if (n_threads < 1) n_threads = 1;
    if (n_threads > 256) n_threads = 256;
    job.stride = n_threads;
    pthread_mutex_init(&job.mu, NULL);
    pthread_t tids[256];
    int32_t started = 0;
    for (int32_t t = 1; t < n_threads; ++t) {
        if (pthread_create(&tids[started], NULL, walk_worker, &job) != 0) break;
        ++started;
    }
    walk_worker(&job); /* also takes the stripes of threads that could not be started */
    for (int32_t t = 0; t < started; ++t) pthread_join(tids[t], NULL);
    pthread_mutex_destroy(&job.mu);
    free(live);
    return job.failed ? -2 : 0;
}

int fsm_oracle_version(void) { return 1; }
