/*
 * router_impl.h — body of the oracle's accumulating router, included by lue_oracle.c once per
 * element type (REAL = float, double).  TEST INFRASTRUCTURE ONLY (see lue_oracle.c).
 *
 * Structure follows ALG/definition/accumulating_router.hpp: per partition an intra phase (row-major
 * scan, walks from every cell whose inflow count is zero, :866-882), walks that stop at sinks,
 * confluences and partition output cells (:525-599), and an inter phase in which (cell, outflow)
 * messages from neighbouring partitions are added to partition input cells; the walk continues from
 * an input cell once its count reaches zero (:984-1010).
 */
#define CAT2(a, b) a##_##b
#define CAT(a, b) CAT2(a, b)
#define FN(name) CAT(name, SFX)

typedef struct {
    int64_t idx;
    REAL value;
} FN(Message);

typedef struct {
    FN(Message) * items;
    int64_t size, cap;
    pthread_mutex_t lock;
    int scheduled;
} FN(Mailbox);

typedef struct {
    int op;
    Grid g;
    const uint8_t* fd;
    int8_t* cnt;        /* router counts, decremented by walks */
    const REAL* a0;     /* external inflow (accu, threshold, fraction) / current outflow (kinematic wave) */
    REAL a0s;
    const REAL* a1;     /* threshold / fraction / lateral inflow */
    REAL a1s;
    const REAL* alpha;
    REAL alphas;
    const REAL* beta;
    REAL betas;
    REAL dt;
    const REAL* dx;
    REAL dxs;
    REAL* out;          /* outflow */
    REAL* rem;          /* remainder (threshold, fraction) */
    FN(Mailbox) * boxes; /* one per partition (threaded mode), or boxes[0] as a FIFO */
    int threaded;
    /* threaded scheduling */
    pthread_mutex_t qlock;
    pthread_cond_t qcond;
    int64_t* ready;
    int64_t ready_head, ready_tail, ready_cap;
    int64_t pending;
    int64_t next_part;
    int done;
} FN(Router);

#define VAL(p, s, i) ((p) ? (p)[i] : (s))

static void FN(box_push)(FN(Mailbox) * b, int64_t idx, REAL v)
{
    if (b->size == b->cap) {
        b->cap = b->cap ? 2 * b->cap : 64;
        b->items = (FN(Message)*)realloc(b->items, (size_t)b->cap * sizeof(FN(Message)));
    }
    b->items[b->size].idx = idx;
    b->items[b->size].value = v;
    b->size++;
}

static inline void FN(mark_no_data)(FN(Router) * R, int64_t i)
{
    R->out[i] = (REAL)NAN;
    if (R->rem) R->rem[i] = (REAL)NAN;
}

/* leave_cell / enter_inter_partition_stream: add upstream outflow, NaN-propagating. */
static inline void FN(add_inflow)(FN(Router) * R, int64_t to, REAL upstream)
{
    if (!isnan(R->out[to])) {
        if (isnan(upstream)) FN(mark_no_data)(R, to);
        else R->out[to] += upstream;
    }
}

static inline void FN(enter_cell)(FN(Router) * R, int64_t i)
{
    REAL* o = &R->out[i];
    if (isnan(*o)) return;
    switch (R->op) {
        case OP_ACCU: {
            REAL e = VAL(R->a0, R->a0s, i);
            if (isnan(e) || !(e >= 0)) *o = (REAL)NAN;
            else *o += e;
            break;
        }
        case OP_THRESHOLD: {
            REAL e = VAL(R->a0, R->a0s, i), t = VAL(R->a1, R->a1s, i);
            if (isnan(e) || isnan(t) || !(e >= 0 && t >= 0)) {
                FN(mark_no_data)(R, i);
            } else {
                *o += e;
                if (*o > t) { R->rem[i] = t; *o -= t; }
                else { R->rem[i] = *o; *o = 0; }
            }
            break;
        }
        case OP_FRACTION: {
            REAL e = VAL(R->a0, R->a0s, i), f = VAL(R->a1, R->a1s, i);
            if (isnan(e) || isnan(f) || !(e >= 0 && f >= 0 && f <= 1)) {
                FN(mark_no_data)(R, i);
            } else {
                *o += e;
                REAL d = f * *o;
                R->rem[i] = *o - d;
                *o = d;
            }
            break;
        }
        case OP_CAPACITY: {  /* ALG/definition/accu_capacity.hpp enter_cell */
            REAL e = VAL(R->a0, R->a0s, i), c = VAL(R->a1, R->a1s, i);
            if (isnan(e) || isnan(c) || !(e >= 0 && c >= 0)) {
                FN(mark_no_data)(R, i);
            } else {
                *o += e;
                R->rem[i] = 0;
                if (*o > c) { R->rem[i] = *o - c; *o = c; }
            }
            break;
        }
        case OP_TRIGGER: {  /* ALG/definition/accu_trigger.hpp enter_cell */
            REAL e = VAL(R->a0, R->a0s, i), t = VAL(R->a1, R->a1s, i);
            if (isnan(e) || isnan(t) || !(e >= 0 && t >= 0)) {
                FN(mark_no_data)(R, i);
            } else {
                *o += e;
                R->rem[i] = 0;
                if (*o < t) { R->rem[i] = *o; *o = 0; }
            }
            break;
        }
        case OP_KINEMATIC_WAVE: {
            REAL qc = VAL(R->a0, R->a0s, i), q = VAL(R->a1, R->a1s, i);
            REAL al = VAL(R->alpha, R->alphas, i), be = VAL(R->beta, R->betas, i);
            REAL dx = VAL(R->dx, R->dxs, i);
            if (isnan(qc) || isnan(q) || isnan(al) || isnan(be) || isnan(R->dt) || isnan(dx) ||
                !(qc >= 0 && q >= 0 && dx > 0)) {
                *o = (REAL)NAN;
            } else {
                *o = ITERATE(*o, qc, q, al, be, R->dt, dx);
            }
            break;
        }
    }
}

/* Walk downstream from cell (r, c) of partition (pr, pc) (accumulating_router.hpp:525-599). */
static void FN(walk)(FN(Router) * R, int64_t pr, int64_t pc, int64_t r, int64_t c)
{
    const Grid* g = &R->g;
    int64_t r0, r1, c0, c1;
    part_rows(g, pr, &r0, &r1);
    part_cols(g, pc, &c0, &c1);
    const int64_t cols = g->cols;
    for (;;) {
        int64_t i = r * cols + c;
        FN(enter_cell)(R, i);
        int dr, dc;
        d8_offset(R->fd[i], &dr, &dc);
        if (dr == 0 && dc == 0) break; /* sink */
        int64_t rd = r + dr, cd = c + dc;
        if (rd < r0 || rd >= r1 || cd < c0 || cd >= c1) {
            /* partition output cell: send to the neighbour partition, if the array has one there */
            if (rd >= 0 && rd < g->rows && cd >= 0 && cd < cols) {
                int64_t j = rd * cols + cd;
                if (R->threaded) {
                    int64_t q = part_of_row(g, rd) * g->npcol + part_of_col(g, cd);
                    FN(Mailbox)* b = &R->boxes[q];
                    pthread_mutex_lock(&R->qlock);
                    R->pending++;
                    pthread_mutex_unlock(&R->qlock);
                    pthread_mutex_lock(&b->lock);
                    FN(box_push)(b, j, R->out[i]);
                    int schedule = !b->scheduled;
                    b->scheduled = 1;
                    pthread_mutex_unlock(&b->lock);
                    if (schedule) {
                        pthread_mutex_lock(&R->qlock);
                        if (R->ready) {
                            if (R->ready_tail - R->ready_head == R->ready_cap) { /* cannot happen: one slot per partition */ }
                            R->ready[R->ready_tail++ % R->ready_cap] = q;
                            pthread_cond_signal(&R->qcond);
                        }
                        pthread_mutex_unlock(&R->qlock);
                    }
                } else {
                    FN(box_push)(&R->boxes[0], j, R->out[i]);
                }
            }
            break;
        }
        int64_t j = rd * cols + cd;
        FN(add_inflow)(R, j, R->out[i]); /* leave_cell */
        r = rd;
        c = cd;
        if (--R->cnt[j] > 0) break; /* confluence */
    }
}

static void FN(intra)(FN(Router) * R, int64_t p)
{
    const Grid* g = &R->g;
    int64_t pr = p / g->npcol, pc = p % g->npcol;
    int64_t r0, r1, c0, c1;
    part_rows(g, pr, &r0, &r1);
    part_cols(g, pc, &c0, &c1);
    /* the ridge test reads the counts as they were before any walk (the reference walks a copy) */
    for (int64_t r = r0; r < r1; ++r) {
        for (int64_t c = c0; c < c1; ++c) {
            int64_t i = r * g->cols + c;
            if (R->fd[i] == U8_NO_DATA) FN(mark_no_data)(R, i);
        }
    }
    int64_t n = (r1 - r0) * (c1 - c0);
    uint8_t* ridge = (uint8_t*)malloc((size_t)n);
    for (int64_t r = r0; r < r1; ++r)
        for (int64_t c = c0; c < c1; ++c)
            ridge[(r - r0) * (c1 - c0) + (c - c0)] =
                R->fd[r * g->cols + c] != U8_NO_DATA && R->cnt[r * g->cols + c] == 0;
    for (int64_t r = r0; r < r1; ++r)
        for (int64_t c = c0; c < c1; ++c)
            if (ridge[(r - r0) * (c1 - c0) + (c - c0)]) FN(walk)(R, pr, pc, r, c);
    free(ridge);
}

/* One arrival at a partition input cell (accumulating_router.hpp:984-1010). */
static void FN(arrive)(FN(Router) * R, int64_t j, REAL v)
{
    const Grid* g = &R->g;
    FN(add_inflow)(R, j, v);
    if (--R->cnt[j] == 0) {
        int64_t r = j / g->cols, c = j % g->cols;
        FN(walk)(R, part_of_row(g, r), part_of_col(g, c), r, c);
    }
}

static void* FN(intra_worker)(void* arg)
{
    FN(Router)* R = (FN(Router)*)arg;
    int64_t np = R->g.nprow * R->g.npcol;
    for (;;) {
        pthread_mutex_lock(&R->qlock);
        int64_t p = R->next_part++;
        pthread_mutex_unlock(&R->qlock);
        if (p >= np) break;
        FN(intra)(R, p);
    }
    return NULL;
}

static void* FN(inter_worker)(void* arg)
{
    FN(Router)* R = (FN(Router)*)arg;
    for (;;) {
        pthread_mutex_lock(&R->qlock);
        while (R->ready_head == R->ready_tail && R->pending > 0 && !R->done)
            pthread_cond_wait(&R->qcond, &R->qlock);
        if (R->ready_head == R->ready_tail) {
            R->done = 1;
            pthread_cond_broadcast(&R->qcond);
            pthread_mutex_unlock(&R->qlock);
            break;
        }
        int64_t p = R->ready[R->ready_head++ % R->ready_cap];
        pthread_mutex_unlock(&R->qlock);

        FN(Mailbox)* b = &R->boxes[p];
        for (;;) {
            pthread_mutex_lock(&b->lock);
            if (b->size == 0) {
                b->scheduled = 0;
                pthread_mutex_unlock(&b->lock);
                break;
            }
            FN(Message)* items = b->items;
            int64_t n = b->size;
            b->items = NULL;
            b->size = b->cap = 0;
            pthread_mutex_unlock(&b->lock);
            for (int64_t k = 0; k < n; ++k) FN(arrive)(R, items[k].idx, items[k].value);
            free(items);
            pthread_mutex_lock(&R->qlock);
            R->pending -= n;
            if (R->pending == 0) pthread_cond_broadcast(&R->qcond);
            pthread_mutex_unlock(&R->qlock);
        }
    }
    return NULL;
}

static int FN(route)(FN(Router) * R, int nthreads)
{
    const Grid* g = &R->g;
    int64_t ncell = g->rows * g->cols, np = g->nprow * g->npcol;
    R->cnt = (int8_t*)malloc((size_t)ncell);
    if (!R->cnt) return -2;
    router_counts(g, R->fd, 1, R->cnt);
    for (int64_t i = 0; i < ncell; ++i) {
        R->out[i] = 0;
        if (R->rem) R->rem[i] = 0;
    }
    R->threaded = nthreads > 1;
    if (!R->threaded) {
        FN(Mailbox) fifo;
        memset(&fifo, 0, sizeof fifo);
        R->boxes = &fifo;
        for (int64_t p = 0; p < np; ++p) FN(intra)(R, p);
        for (int64_t k = 0; k < fifo.size; ++k) FN(arrive)(R, fifo.items[k].idx, fifo.items[k].value);
        free(fifo.items);
    } else {
        R->boxes = (FN(Mailbox)*)calloc((size_t)np, sizeof(FN(Mailbox)));
        for (int64_t p = 0; p < np; ++p) pthread_mutex_init(&R->boxes[p].lock, NULL);
        pthread_mutex_init(&R->qlock, NULL);
        pthread_cond_init(&R->qcond, NULL);
        R->ready = NULL; /* phase 1 only fills mailboxes */
        R->pending = 0;
        R->next_part = 0;
        pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
        for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, FN(intra_worker), R);
        for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
        /* phase 2: every partition with mail is ready */
        R->ready_cap = np + 1;
        R->ready = (int64_t*)malloc(sizeof(int64_t) * (size_t)R->ready_cap);
        R->ready_head = R->ready_tail = 0;
        for (int64_t p = 0; p < np; ++p) {
            R->boxes[p].scheduled = R->boxes[p].size > 0;
            if (R->boxes[p].size > 0) R->ready[R->ready_tail++] = p;
        }
        R->done = 0;
        for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, FN(inter_worker), R);
        for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
        for (int64_t p = 0; p < np; ++p) {
            free(R->boxes[p].items);
            pthread_mutex_destroy(&R->boxes[p].lock);
        }
        free(R->boxes);
        free(R->ready);
        free(th);
        pthread_mutex_destroy(&R->qlock);
        pthread_cond_destroy(&R->qcond);
    }
    free(R->cnt);
    return 0;
}

static int FN(setup)(FN(Router) * R, int op, const uint8_t* fd, int64_t rows, int64_t cols, int64_t prow,
                     int64_t pcol)
{
    memset(R, 0, sizeof *R);
    R->op = op;
    R->fd = fd;
    return grid_init(&R->g, rows, cols, prow, pcol);
}

/* value_policies::accu (ALG/value_policies/accu.hpp:33-55).  ext == NULL: scalar ext_scalar. */
int FN(lue_oracle_accu)(const uint8_t* fd, int64_t rows, int64_t cols, int64_t prow, int64_t pcol,
                        const REAL* ext, REAL ext_scalar, REAL* out, int nthreads)
{
    FN(Router) R;
    if (FN(setup)(&R, OP_ACCU, fd, rows, cols, prow, pcol)) return -1;
    R.a0 = ext; R.a0s = ext_scalar; R.out = out;
    return FN(route)(&R, nthreads);
}

/* value_policies::accu_threshold: (flux, state) = (out, rem). */
int FN(lue_oracle_accu_threshold)(const uint8_t* fd, int64_t rows, int64_t cols, int64_t prow, int64_t pcol,
                                  const REAL* ext, REAL ext_scalar, const REAL* thr, REAL thr_scalar,
                                  REAL* flux, REAL* state, int nthreads)
{
    FN(Router) R;
    if (FN(setup)(&R, OP_THRESHOLD, fd, rows, cols, prow, pcol)) return -1;
    R.a0 = ext; R.a0s = ext_scalar; R.a1 = thr; R.a1s = thr_scalar; R.out = flux; R.rem = state;
    return FN(route)(&R, nthreads);
}

/* value_policies::accu_fraction: (flux, state) = (out, rem). */
int FN(lue_oracle_accu_fraction)(const uint8_t* fd, int64_t rows, int64_t cols, int64_t prow, int64_t pcol,
                                 const REAL* ext, REAL ext_scalar, const REAL* frac, REAL frac_scalar,
                                 REAL* flux, REAL* state, int nthreads)
{
    FN(Router) R;
    if (FN(setup)(&R, OP_FRACTION, fd, rows, cols, prow, pcol)) return -1;
    R.a0 = ext; R.a0s = ext_scalar; R.a1 = frac; R.a1s = frac_scalar; R.out = flux; R.rem = state;
    return FN(route)(&R, nthreads);
}

/* value_policies::accu_capacity: (outflow, remainder); domain inflow >= 0 && capacity >= 0
   (ALG/value_policies/accu_capacity.hpp:15-18). */
int FN(lue_oracle_accu_capacity)(const uint8_t* fd, int64_t rows, int64_t cols, int64_t prow, int64_t pcol,
                                 const REAL* ext, REAL ext_scalar, const REAL* cap, REAL cap_scalar,
                                 REAL* outflow, REAL* remainder, int nthreads)
{
    FN(Router) R;
    if (FN(setup)(&R, OP_CAPACITY, fd, rows, cols, prow, pcol)) return -1;
    R.a0 = ext; R.a0s = ext_scalar; R.a1 = cap; R.a1s = cap_scalar; R.out = outflow; R.rem = remainder;
    return FN(route)(&R, nthreads);
}

/* value_policies::accu_trigger: (outflow, remainder); domain inflow >= 0 && trigger >= 0
   (ALG/value_policies/accu_trigger.hpp:15-18). */
int FN(lue_oracle_accu_trigger)(const uint8_t* fd, int64_t rows, int64_t cols, int64_t prow, int64_t pcol,
                                const REAL* ext, REAL ext_scalar, const REAL* trig, REAL trig_scalar,
                                REAL* outflow, REAL* remainder, int nthreads)
{
    FN(Router) R;
    if (FN(setup)(&R, OP_TRIGGER, fd, rows, cols, prow, pcol)) return -1;
    R.a0 = ext; R.a0s = ext_scalar; R.a1 = trig; R.a1s = trig_scalar; R.out = outflow; R.rem = remainder;
    return FN(route)(&R, nthreads);
}

/* value_policies::kinematic_wave (ALG/value_policies/kinematic_wave.hpp:43-91): one time step. */
int FN(lue_oracle_kinematic_wave)(const uint8_t* fd, int64_t rows, int64_t cols, int64_t prow, int64_t pcol,
                                  const REAL* qcur, REAL qcur_s, const REAL* lateral, REAL lateral_s,
                                  const REAL* alpha, REAL alpha_s, const REAL* beta, REAL beta_s, REAL dt,
                                  const REAL* dx, REAL dx_s, REAL* out, int nthreads)
{
    FN(Router) R;
    if (FN(setup)(&R, OP_KINEMATIC_WAVE, fd, rows, cols, prow, pcol)) return -1;
    R.a0 = qcur; R.a0s = qcur_s; R.a1 = lateral; R.a1s = lateral_s;
    R.alpha = alpha; R.alphas = alpha_s; R.beta = beta; R.betas = beta_s; R.dt = dt;
    R.dx = dx; R.dxs = dx_s; R.out = out;
    return FN(route)(&R, nthreads);
}

#undef VAL
#undef FN
#undef CAT
#undef CAT2
