/* Body of the C restatement of the tinyfluids step, included twice by
 * fluid_ref.c: once with R=float (the reference's float32 scheme) and once
 * with R=double (the FP64 oracle).  TEST INFRASTRUCTURE ONLY.
 *
 * Every expression keeps the evaluation order of the reference
 * (tinyfluids/jax_tinyfluids/fluid.py) so that, compiled with
 * -ffp-contract=off, the float build is bit-identical to oracle/fluid_np.py.
 * Layout: [5][nx][ny][nz], z contiguous (fluid.py:10-22).
 */

/* fluid.py:47-53 and :231-237: E = p/(g-1) + 0.5*rho*sqrt(|u|^2)**2 */
static inline R FN(energy)(R rho, R vx, R vy, R vz, R p, R g)
{
    R ut = SQRT((vx * vx + vy * vy) + vz * vz);
    return p / (g - (R)1) + ((R)0.5 * rho) * (ut * ut);
}

/* fluid.py:106-117: c = sqrt(gamma*p/rho) */
static inline R FN(sound)(R rho, R p, R g) { return SQRT((g * p) / rho); }

/* Per-cell quantities of one line, computed once per cell:
 * conserved U (fluid.py:44-65), Euler flux F along velocity index vel
 * (fluid.py:225-257), u = v_vel and c. */
typedef struct { R U[5], F[5], u, c; } FN(cell_t);

static inline void FN(derive)(const R w[5], int vel, R g, FN(cell_t) *o)
{
    R rho = w[0], p = w[4];
    R E = FN(energy)(rho, w[1], w[2], w[3], p, g);
    R ud = w[vel];
    o->U[0] = rho;
    o->U[1] = rho * w[1];
    o->U[2] = rho * w[2];
    o->U[3] = rho * w[3];
    o->U[4] = E;
    o->F[0] = ud * rho;
    o->F[1] = ud * (w[1] * rho);
    o->F[2] = ud * (w[2] * rho);
    o->F[3] = ud * (w[3] * rho);
    o->F[4] = ud * (p + E);
    o->F[vel] = o->F[vel] + p;
    o->u = ud;
    o->c = FN(sound)(rho, p, g);
}

/* fluid.py:282-303: HLL flux at the interface between L (left) and R. */
static inline void FN(hll)(const FN(cell_t) *L, const FN(cell_t) *Rc, R out[5])
{
    R a = L->u + L->c, b = Rc->u + Rc->c;
    R sp = a > b ? a : b;
    sp = sp > (R)0 ? sp : (R)0;
    R a2 = L->u - L->c, b2 = Rc->u - Rc->c;
    R sm = a2 < b2 ? a2 : b2;
    sm = sm < (R)0 ? sm : (R)0;
    R smsp = sm * sp, den = sp - sm;
    for (int k = 0; k < 5; ++k)
        out[k] = ((sp * L->F[k] - sm * Rc->F[k]) + smsp * (Rc->U[k] - L->U[k])) / den;
}

/* fluid.py:85-101: primitive from conserved. */
static inline void FN(prim)(const R U[5], R g, R w[5])
{
    R rho = U[0], E = U[4];
    R ux = U[1] / rho, uy = U[2] / rho, uz = U[3] / rho;
    R u = SQRT((ux * ux + uy * uy) + uz * uz);
    w[0] = rho;
    w[1] = ux;
    w[2] = uy;
    w[3] = uz;
    w[4] = ((g - (R)1) * rho) * (E / rho - (R)0.5 * (u * u));
}

/* fluid.py:508-557: one periodic sweep along axis (0=x, 1=y, 2=z), in place.
 * Lines along the axis are independent; each is gathered, swept and
 * scattered by one thread. */
static void FN(sweep)(R *W, int nx, int ny, int nz, R dx, R dt, R g, int axis)
{
    const long long n3 = (long long)nx * ny * nz;
    const int len = axis == 0 ? nx : (axis == 1 ? ny : nz);
    const long long stride = axis == 0 ? (long long)ny * nz : (axis == 1 ? nz : 1);
    const long long nlines = n3 / len;
    const int vel = axis + 1;
    const R inv_dx = (R)1 / dx;
#pragma omp parallel
    {
        FN(cell_t) *cells = (FN(cell_t) *)malloc(sizeof(FN(cell_t)) * (size_t)len);
        R *flux = (R *)malloc(sizeof(R) * 5 * (size_t)len);
#pragma omp for schedule(static)
        for (long long line = 0; line < nlines; ++line) {
            long long base;
            if (axis == 0) base = line;                       /* (y,z) plane index */
            else if (axis == 1) base = (line / nz) * (long long)ny * nz + line % nz;
            else base = line * nz;
            for (int i = 0; i < len; ++i) {
                R w[5];
                for (int v = 0; v < 5; ++v) w[v] = W[v * n3 + base + i * stride];
                FN(derive)(w, vel, g, &cells[i]);
            }
            /* flux[i] is the flux at the face between cells i-1 and i (roll +1) */
            for (int i = 0; i < len; ++i)
                FN(hll)(&cells[i == 0 ? len - 1 : i - 1], &cells[i], &flux[5 * i]);
            for (int i = 0; i < len; ++i) {
                const R *fl = &flux[5 * i];
                const R *fh = &flux[5 * (i + 1 == len ? 0 : i + 1)];
                R U[5], w[5];
                for (int k = 0; k < 5; ++k)
                    U[k] = cells[i].U[k] + (inv_dx * (fl[k] - fh[k])) * dt;
                FN(prim)(U, g, w);
                for (int v = 0; v < 5; ++v) W[v * n3 + base + i * stride] = w[v];
            }
        }
        free(cells);
        free(flux);
    }
}

/* fluid.py:317-413: open boundaries with one ghost cell, x then y then z,
 * left then right, each a slab copy. */
static void FN(open_boundaries)(R *W, int nx, int ny, int nz)
{
    const long long n3 = (long long)nx * ny * nz;
    const int dims[3] = {nx, ny, nz};
    const long long strides[3] = {(long long)ny * nz, nz, 1};
    for (int axis = 0; axis < 3; ++axis) {
        const int len = dims[axis];
        const long long st = strides[axis];
        const long long nlines = n3 / len;
        for (int side = 0; side < 2; ++side) {
            int set = side == 0 ? 0 : len - 1;
            int get = side == 0 ? 1 : len - 2;
#pragma omp parallel for schedule(static)
            for (long long line = 0; line < nlines; ++line) {
                long long base;
                if (axis == 0) base = line;
                else if (axis == 1) base = (line / nz) * (long long)ny * nz + line % nz;
                else base = line * nz;
                for (int v = 0; v < 5; ++v)
                    W[v * n3 + base + set * st] = W[v * n3 + base + get * st];
            }
        }
    }
}

/* fluid.py:427-504: C_CFL*dx / max over axes and periodic interfaces of
 * max(|S+|, |S-|). */
R FN(orc_cfl_time_step)(const R *W, int nx, int ny, int nz, R dx, R g, R cfl)
{
    const long long n3 = (long long)nx * ny * nz;
    R axmax[3];
    const int dims[3] = {nx, ny, nz};
    const long long strides[3] = {(long long)ny * nz, nz, 1};
    for (int axis = 0; axis < 3; ++axis) {
        const int vel = axis + 1;
        R best_p = 0, best_m = 0;
#pragma omp parallel
        {
            R lp = 0, lm = 0;
#pragma omp for schedule(static)
            for (long long i = 0; i < n3; ++i) {
                long long ia = (i / strides[axis]) % dims[axis];
                long long il = ia == 0 ? i + (dims[axis] - 1) * strides[axis] : i - strides[axis];
                R rl = W[il], ul = W[vel * n3 + il], pl = W[4 * n3 + il];
                R rr = W[i], ur = W[vel * n3 + i], pr = W[4 * n3 + i];
                R cl = FN(sound)(rl, pl, g), cr = FN(sound)(rr, pr, g);
                R a = ul + cl, b = ur + cr;
                R sp = a > b ? a : b;
                sp = sp > (R)0 ? sp : (R)0;
                R a2 = ul - cl, b2 = ur - cr;
                R sm = a2 < b2 ? a2 : b2;
                sm = sm < (R)0 ? sm : (R)0;
                R asp = sp < 0 ? -sp : sp, asm_ = sm < 0 ? -sm : sm;
                if (asp > lp) lp = asp;
                if (asm_ > lm) lm = asm_;
            }
#pragma omp critical
            {
                if (lp > best_p) best_p = lp;
                if (lm > best_m) best_m = lm;
            }
        }
        axmax[axis] = best_p > best_m ? best_p : best_m;
    }
    R m = axmax[0] > axmax[1] ? axmax[0] : axmax[1];
    m = m > axmax[2] ? m : axmax[2];
    return (cfl * dx) / m;
}

/* fluid.py:562-578, in place. */
void FN(orc_evolve_state)(R *W, int nx, int ny, int nz, R dx, R dt, R g, int handle_boundaries)
{
    if (handle_boundaries) FN(open_boundaries)(W, nx, ny, nz);
    FN(sweep)(W, nx, ny, nz, dx, dt, g, 0);
    FN(sweep)(W, nx, ny, nz, dx, dt, g, 1);
    FN(sweep)(W, nx, ny, nz, dx, dt, g, 2);
}

/* time_integration.py:63-92: while t < t_final: dt = cfl(W); W = step(W, dt);
 * t += dt (in R); it += 1.  fixed_dt > 0 replaces the CFL dt; max_steps >= 0
 * bounds the loop.  dts (optional, length >= max_steps) receives each dt.
 * Returns the number of steps taken; *t_out gets the final time. */
int FN(orc_time_integration)(R *W, int nx, int ny, int nz, R dx, R t_final, R g,
                             int handle_boundaries, R cfl, R fixed_dt,
                             int max_steps, R *dts, R *t_out)
{
    R t = 0;
    int it = 0;
    while (t < t_final) {
        if (max_steps >= 0 && it >= max_steps) break;
        R dt = fixed_dt > 0 ? fixed_dt : FN(orc_cfl_time_step)(W, nx, ny, nz, dx, g, cfl);
        FN(orc_evolve_state)(W, nx, ny, nz, dx, dt, g, handle_boundaries);
        if (dts) dts[it] = dt;
        t = t + dt;
        it += 1;
    }
    if (t_out) *t_out = t;
    return it;
}
