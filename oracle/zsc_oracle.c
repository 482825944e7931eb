/*
 * zsc_oracle.c -- FP64 CPU oracle for the Zheng-Shu-Chew (ZSC) free-energy
 * multiphase lattice Boltzmann step (D3Q7 order parameter f + D3Q19 momentum g).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
 * smoke check and the CPU-baseline leg of bench.py call it; the product path
 * (liblbm_gb300.so) never links or calls it.
 *
 * It restates, in double precision and on a fully periodic box, the update that
 * carlosrosales/lbm_bench_gpu performs with seven kernels and three host-staged
 * halo exchanges per step.  Every function cites the reference lines it follows
 * (paths relative to the reference project root).  Naming follows the
 * reference: f = D3Q7 order-parameter distribution (relaxed with tauPhi),
 * g = D3Q19 momentum distribution (relaxed with tauRho), rho = ZSC mean
 * density n.
 *
 * Layout: idx = x + nx*(y + ny*z), x fastest, z in [0, nz).  The reference
 * stores the same interior node at plane k = z + 1 between two ghost planes
 * (src/vgrid.c:38-52 with one rank: zl = 1, zu = zmax, NZ = zmax + 2).  With one
 * rank the three halo exchanges (src/mpiupdate*.c:34-41 with top = bot = self)
 * are exactly periodic wrap in z, which is what this file does with index
 * arithmetic.  The only place the ghost planes are not periodic copies is the
 * initial equilibrium (src/init.c:39-59 fills them from the bubble geometry and
 * src/init_f.cu, src/init_g.cu read them through the Laplacian); zo_init takes
 * those two planes as an optional argument.
 *
 * Build: cc -O2 -fopenmp -fPIC -shared zsc_oracle.c -o libzsc_oracle.so -lm
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>

#ifdef _OPENMP
#include <omp.h>
#endif

/* Lattice weights and forcing weights, src/constants.h:52-59. */
#define ZO_W0 (1.0 / 3.0)
#define ZO_W1 (1.0 / 18.0)
#define ZO_W2 (1.0 / 36.0)
#define ZO_WC0 1.0
#define ZO_WC1 (1.0 / 6.0)
#define ZO_WC2 (1.0 / 12.0)

typedef struct {
    /* inputs (properties.in values, promoted from float) */
    double rhoL, rhoH, tauRho, tauPhi, width, sigma, Gamma, Eo, rc0;
    /* derived, src/paramread.c:141-170 */
    double phiStar, phiStarSq, invTauRho, invTauRhoOne, invTauRhoHalf;
    double eta, eta2, invEta2, invTauPhi, invTauPhiOne;
    double alpha, alpha4, kappa, gravity, grav;
    double K0, K1, K2, KC0, KC1, KC2;
} zo_const;

typedef struct zo_ctx {
    int nx, ny, nz;
    long n;
    zo_const c;
    long steps;
    double *f[7], *fp[7];     /* streamed / post-collision (reference lower / upper half) */
    double *g[19], *gp[19];
    double *phi, *rho, *ux, *uy, *uz;   /* moment arrays as the reference holds them */
    /* Heavy-node log (test aid for finite differences, see zo_heavy_mask):
     * one byte per node and collision, H(phi > 0) of each step. */
    unsigned char *heavy_log;
    long heavy_cap, heavy_pos;
    int heavy_mode;               /* 0 phi > 0, 1 record, 2 replay */
    /* z-slab of a larger periodic box (zo_slab_create): no z wrap; the planes
     * just below and above the slab come from its neighbours, phi after the
     * moments (2 planes) and the post-collision P, Q after the collision
     * (2 x 26 planes: side, then f 0..6, g 0..18). */
    int slab;
    double *phi_ghost, *post_ghost;
    /* Storage-rounding emulation (precision studies, zo_set_rounding): the
     * post-collision f_0, f_1..f_6 and g sets rounded after every collision
     * to the formats a GPU build stores them in. */
    int round_f0, round_f, round_g;
    double f_scale, g_scale, g_shift[19];
} zo_ctx;

static inline long zo_idx(const zo_ctx *s, int x, int y, int z)
{
    return (long)x + (long)s->nx * ((long)y + (long)s->ny * (long)z);
}

static inline int wrap(int a, int n) { return a < 0 ? a + n : (a >= n ? a - n : a); }

/* Derived constants: src/paramread.c:141-170 (same formulas, in double). */
static void zo_derive(zo_const *c)
{
    c->phiStar = 0.5 * (c->rhoH - c->rhoL);
    c->phiStarSq = c->phiStar * c->phiStar;
    c->invTauRho = 1.0 / c->tauRho;
    c->invTauRhoOne = 1.0 - c->invTauRho;
    c->invTauRhoHalf = 1.0 - 0.5 * c->invTauRho;
    c->eta = 1.0 / (c->tauPhi + 0.5);
    c->eta2 = 1.0 - c->eta;
    c->invEta2 = 0.5 / (1.0 - c->eta);
    c->invTauPhi = 1.0 / c->tauPhi;
    c->invTauPhiOne = 1.0 - c->invTauPhi;
    c->alpha = 0.75 * c->sigma / (c->width * c->phiStarSq * c->phiStarSq);
    c->alpha4 = 4.0 * c->alpha;
    c->kappa = (c->width * c->phiStar) * (c->width * c->phiStar) * c->alpha * 0.5;
    c->gravity = 0.25 * c->Eo * c->sigma / ((c->rhoH - c->rhoL) * c->rc0 * c->rc0);
    c->grav = 2.0 * c->phiStar * c->gravity;
    c->K0 = c->invTauRho * ZO_W0;
    c->K1 = c->invTauRho * ZO_W1;
    c->K2 = c->invTauRho * ZO_W2;
    c->KC0 = c->invTauRhoHalf * ZO_WC0;
    c->KC1 = c->invTauRhoHalf * ZO_WC1;
    c->KC2 = c->invTauRhoHalf * ZO_WC2;
}

/* prm = {rhoL, rhoH, tauRho, tauPhi, width, sigma, Gamma, Eo, rc0} */
zo_ctx *zo_create(int nx, int ny, int nz, const double *prm)
{
    if (nx < 3 || ny < 3 || nz < 3) return NULL;
    zo_ctx *s = (zo_ctx *)calloc(1, sizeof(zo_ctx));
    if (!s) return NULL;
    s->nx = nx; s->ny = ny; s->nz = nz;
    s->n = (long)nx * ny * nz;
    s->c.rhoL = prm[0]; s->c.rhoH = prm[1]; s->c.tauRho = prm[2]; s->c.tauPhi = prm[3];
    s->c.width = prm[4]; s->c.sigma = prm[5]; s->c.Gamma = prm[6]; s->c.Eo = prm[7];
    s->c.rc0 = prm[8];
    zo_derive(&s->c);
    int ok = 1;
    for (int i = 0; i < 7; i++) {
        s->f[i] = (double *)malloc(sizeof(double) * s->n);
        s->fp[i] = (double *)malloc(sizeof(double) * s->n);
        ok &= s->f[i] && s->fp[i];
    }
    for (int i = 0; i < 19; i++) {
        s->g[i] = (double *)malloc(sizeof(double) * s->n);
        s->gp[i] = (double *)malloc(sizeof(double) * s->n);
        ok &= s->g[i] && s->gp[i];
    }
    s->phi = (double *)malloc(sizeof(double) * s->n);
    s->rho = (double *)malloc(sizeof(double) * s->n);
    s->ux = (double *)malloc(sizeof(double) * s->n);
    s->uy = (double *)malloc(sizeof(double) * s->n);
    s->uz = (double *)malloc(sizeof(double) * s->n);
    ok &= s->phi && s->rho && s->ux && s->uy && s->uz;
    if (!ok) {
        extern void zo_destroy(zo_ctx *);
        zo_destroy(s);
        return NULL;
    }
    return s;
}

void zo_destroy(zo_ctx *s)
{
    if (!s) return;
    for (int i = 0; i < 7; i++) { free(s->f[i]); free(s->fp[i]); }
    for (int i = 0; i < 19; i++) { free(s->g[i]); free(s->gp[i]); }
    free(s->phi); free(s->rho); free(s->ux); free(s->uy); free(s->uz);
    free(s->heavy_log);
    free(s->phi_ghost);
    free(s->post_ghost);
    free(s);
}

/* out = {phiStar, phiStarSq, invTauRho, invTauRhoOne, invTauRhoHalf, eta, eta2,
 *        invEta2, invTauPhi, invTauPhiOne, alpha, alpha4, kappa, gravity, grav,
 *        K0, K1, K2, KC0, KC1, KC2} */
void zo_constants(const zo_ctx *s, double *out)
{
    const zo_const *c = &s->c;
    double v[21] = {c->phiStar, c->phiStarSq, c->invTauRho, c->invTauRhoOne, c->invTauRhoHalf,
                    c->eta, c->eta2, c->invEta2, c->invTauPhi, c->invTauPhiOne,
                    c->alpha, c->alpha4, c->kappa, c->gravity, c->grav,
                    c->K0, c->K1, c->K2, c->KC0, c->KC1, c->KC2};
    memcpy(out, v, sizeof(v));
}

long zo_steps(const zo_ctx *s) { return s->steps; }

/*
 * Bubble initial condition, src/init.c:39-59: phi = -phiStar everywhere, then
 * for each bubble in file order, nodes with R <= Rc + width take
 * phi = phiStar * tanh(2 (Rc - R) / width) (last writer wins, no minimum image).
 * x, y are 0-based, the reference z coordinate is 1-based; the output holds the
 * two ghost planes too: plane kk in [0, nz+1] is reference z = kk.
 * Membership (R <= Rc + width) is decided in float arithmetic, as the reference
 * does, so that nodes on the shell boundary fall on the same side; the value
 * is then evaluated in double.
 */
void zo_bubble_phi(const zo_ctx *s, const float *bubbles, int nb, double *phi_g)
{
    const int nx = s->nx, ny = s->ny, nzg = s->nz + 2;
    const long ng = (long)nx * ny * nzg;
    const double phiStar = s->c.phiStar, width = s->c.width;
    const float widthf = (float)width;
#pragma omp parallel for schedule(static)
    for (long q = 0; q < ng; q++) phi_g[q] = -phiStar;
    /* Bubbles in file order over the nodes of their bounding boxes (two nodes
     * of margin around Rc + width, far more than the float rounding of R), so
     * a later bubble overwrites an earlier one exactly where the reference's
     * loop over all bubbles per node would. */
    for (int m = 0; m < nb; m++) {
        const float xc = bubbles[4 * m + 0], yc = bubbles[4 * m + 1];
        const float zc = bubbles[4 * m + 2], rc = bubbles[4 * m + 3];
        const double reach = (double)rc + width + 2.0;
        int lo[3], hi[3];
        const float cc[3] = {xc, yc, zc};
        const int ext[3] = {nx, ny, nzg};
        for (int a = 0; a < 3; a++) {
            double l = floor((double)cc[a] - reach), h = ceil((double)cc[a] + reach);
            lo[a] = l < 0 ? 0 : (l > ext[a] ? ext[a] : (int)l);
            hi[a] = h > ext[a] - 1 ? ext[a] - 1 : (h < -1 ? -1 : (int)h);
        }
#pragma omp parallel for schedule(static)
        for (int kk = lo[2]; kk <= hi[2]; kk++) {
            for (int j = lo[1]; j <= hi[1]; j++) {
                for (int i = lo[0]; i <= hi[0]; i++) {
                    volatile float dxf = (float)i - xc;
                    volatile float dyf = (float)j - yc;
                    volatile float dzf = (float)kk - zc;
                    volatile float sx = dxf * dxf, sy = dyf * dyf, sz = dzf * dzf;
                    volatile float ssum = sx + sy;
                    ssum = ssum + sz;
                    const float Rf = sqrtf(ssum);
                    if (Rf <= rc + widthf) {
                        const double dx = (double)i - xc, dy = (double)j - yc, dz = (double)kk - zc;
                        const double R = sqrt(dx * dx + dy * dy + dz * dz);
                        phi_g[(long)i + (long)nx * ((long)j + (long)ny * kk)] =
                            phiStar * tanh(2.0 * ((double)rc - R) / width);
                    }
                }
            }
        }
    }
}

/* phi at (x, y, z) with periodic x, y and, in z, either periodic wrap or the
 * supplied ghost planes (ghost[0..nx*ny) = plane below z = 0, ghost[nx*ny..) =
 * plane above z = nz-1). */
static inline double phi_at(const zo_ctx *s, const double *phi, const double *ghost, int x, int y, int z)
{
    x = wrap(x, s->nx);
    y = wrap(y, s->ny);
    if (z < 0 || z >= s->nz) {
        if (ghost) {
            const long p = (long)x + (long)s->nx * y;
            return z < 0 ? ghost[p] : ghost[(long)s->nx * s->ny + p];
        }
        z = wrap(z, s->nz);
    }
    return phi[zo_idx(s, x, y, z)];
}

/* The 19-point isotropic stencil of the reference: Laplacian
 * (src/collision_f.cu:61-70) and gradient (src/collision_f.cu:78-94). */
static inline void stencil(const zo_ctx *s, const double *phi, const double *ghost, int x, int y, int z,
                           double *lap, double *gx, double *gy, double *gz)
{
#define P(dx, dy, dz) phi_at(s, phi, ghost, x + (dx), y + (dy), z + (dz))
    const double c = P(0, 0, 0);
    const double e = P(1, 0, 0), w = P(-1, 0, 0), n = P(0, 1, 0), so = P(0, -1, 0);
    const double t = P(0, 0, 1), b = P(0, 0, -1);
    const double en = P(1, 1, 0), ws = P(-1, -1, 0), es = P(1, -1, 0), wn = P(-1, 1, 0);
    const double et = P(1, 0, 1), wb = P(-1, 0, -1), eb = P(1, 0, -1), wt = P(-1, 0, 1);
    const double nt = P(0, 1, 1), sb = P(0, -1, -1), nb = P(0, 1, -1), st = P(0, -1, 1);
#undef P
    *lap = (en + ws + es + wn + et + wb + eb + wt + nt + sb + nb + st
            + 2.0 * (e + w + n + so + t + b - 12.0 * c)) / 6.0;
    *gx = (2.0 * (e - w) + en - ws + es - wn + et - wb + eb - wt) / 12.0;
    *gy = (2.0 * (n - so) + en - ws + wn - es + nt - sb + nb - st) / 12.0;
    *gz = (2.0 * (t - b) + et - wb + wt - eb + nt - sb + st - nb) / 12.0;
}

/*
 * Initial equilibrium at rest: src/init_f.cu:42-79 and src/init_g.cu:46-93.
 * Also fills the moment arrays with the given fields (src/main.cu copies the
 * host phi, rho, ux, uy, uz to the device before init_f/init_g).  The initial
 * velocity does not enter the distributions (both kernels build the at-rest
 * equilibrium).  ghost: NULL for periodic z, else the two planes (see phi_at).
 */
void zo_init(zo_ctx *s, const double *phi, const double *rho, const double *ux, const double *uy,
             const double *uz, const double *ghost)
{
    const zo_const *c = &s->c;
    s->heavy_pos = 0;
    memcpy(s->phi, phi, sizeof(double) * s->n);
    memcpy(s->rho, rho, sizeof(double) * s->n);
    memcpy(s->ux, ux, sizeof(double) * s->n);
    memcpy(s->uy, uy, sizeof(double) * s->n);
    memcpy(s->uz, uz, sizeof(double) * s->n);
#pragma omp parallel for schedule(static)
    for (int z = 0; z < s->nz; z++) {
        for (int y = 0; y < s->ny; y++) {
            for (int x = 0; x < s->nx; x++) {
                const long id = zo_idx(s, x, y, z);
                double lap, gx, gy, gz;
                stencil(s, s->phi, ghost, x, y, z, &lap, &gx, &gy, &gz);
                const double ph = s->phi[id], rh = s->rho[id];
                const double mu = c->alpha4 * ph * (ph * ph - c->phiStarSq) - c->kappa * lap;
                const double Af = 0.5 * c->Gamma * mu;
                s->f[0][id] = ph - 3.0 * c->Gamma * mu;
                for (int i = 1; i < 7; i++) s->f[i][id] = Af;
                const double Ag1 = ZO_W1 * (3.0 * ph * mu + rh);
                const double Ag2 = ZO_W2 * (3.0 * ph * mu + rh);
                s->g[0][id] = ZO_W0 * (rh - 6.0 * ph * mu);
                for (int i = 1; i < 7; i++) s->g[i][id] = Ag1;
                for (int i = 7; i < 19; i++) s->g[i][id] = Ag2;
            }
        }
    }
    s->steps = 0;
}

/* update_phi, update_rho, update_velocity: src/update_phi.cu:40-44,
 * src/update_rho.cu:44-51, src/update_velocity.cu:45-61. */
static void zo_moments_update(zo_ctx *s)
{
    double **f = s->f, **g = s->g;
#pragma omp parallel for schedule(static)
    for (long id = 0; id < s->n; id++) {
        s->phi[id] = f[0][id] + f[1][id] + f[2][id] + f[3][id] + f[4][id] + f[5][id] + f[6][id];
        double r = 0.0;
        for (int i = 0; i < 19; i++) r += g[i][id];
        s->rho[id] = r;
        const double inv = 1.0 / r;
        s->ux[id] = (g[1][id] - g[2][id] + g[7][id] - g[8][id] + g[9][id] - g[10][id]
                     + g[11][id] - g[12][id] + g[13][id] - g[14][id]) * inv;
        s->uy[id] = (g[3][id] - g[4][id] + g[7][id] - g[8][id] - g[9][id] + g[10][id]
                     + g[15][id] - g[16][id] + g[17][id] - g[18][id]) * inv;
        s->uz[id] = (g[5][id] - g[6][id] + g[11][id] - g[12][id] - g[13][id] + g[14][id]
                     + g[15][id] - g[16][id] - g[17][id] + g[18][id]) * inv;
    }
}

/* collision_f (src/collision_f.cu:44-116) and collision_g
 * (src/collision_g.cu:49-196), both on every node, into fp / gp. */
static void zo_collide(zo_ctx *s, double grav)
{
    const zo_const *c = &s->c;
    unsigned char *heavy_log = NULL;
    if (s->heavy_mode && s->heavy_log && s->heavy_pos + s->n <= s->heavy_cap) {
        heavy_log = s->heavy_log + s->heavy_pos;
        s->heavy_pos += s->n;
    }
#pragma omp parallel for schedule(static)
    for (int z = 0; z < s->nz; z++) {
        for (int y = 0; y < s->ny; y++) {
            for (int x = 0; x < s->nx; x++) {
                const long id = zo_idx(s, x, y, z);
                double lap, gx, gy, gz;
                stencil(s, s->phi, s->phi_ghost, x, y, z, &lap, &gx, &gy, &gz);
                const double ph = s->phi[id], rh = s->rho[id];
                const double mu = c->alpha4 * ph * (ph * ph - c->phiStarSq) - c->kappa * lap;
                const double Fx = mu * gx, Fy = mu * gy;
                double Fz = mu * gz;
                int heavy = ph > 0.0;
                if (heavy_log) {
                    if (s->heavy_mode == 2) heavy = heavy_log[id];
                    else heavy_log[id] = (unsigned char)heavy;
                }
                if (heavy) Fz += grav;
                const double ux = s->ux[id] + 0.5 * Fx / rh;
                const double uy = s->uy[id] + 0.5 * Fy / rh;
                const double uz = s->uz[id] + 0.5 * Fz / rh;

                /* D3Q7, order parameter */
                const double Af = 0.5 * c->Gamma * c->invTauPhi * mu;
                const double Cf = c->invTauPhi * c->invEta2 * ph;
                const double a = c->invTauPhiOne;
                s->fp[0][id] = a * s->f[0][id] - 6.0 * Af + c->invTauPhi * ph;
                s->fp[1][id] = a * s->f[1][id] + Af + Cf * ux;
                s->fp[2][id] = a * s->f[2][id] + Af - Cf * ux;
                s->fp[3][id] = a * s->f[3][id] + Af + Cf * uy;
                s->fp[4][id] = a * s->f[4][id] + Af - Cf * uy;
                s->fp[5][id] = a * s->f[5][id] + Af + Cf * uz;
                s->fp[6][id] = a * s->f[6][id] + Af - Cf * uz;

                /* D3Q19, momentum with forcing */
                const double b = c->invTauRhoOne;
                const double UF = ux * Fx + uy * Fy + uz * Fz;
                const double usq = ux * ux + uy * uy + uz * uz;
                const double temp1 = c->K1 * (3.0 * ph * mu + rh * (1.0 - 1.5 * usq));
                const double vx = 3.0 * ux, vy = 3.0 * uy, vz = 3.0 * uz;
                const double vsq = vx * vx + vy * vy + vz * vz;
                double **g = s->g, **gp = s->gp;
                gp[0][id] = b * g[0][id] + c->K0 * (rh - 6.0 * ph * mu - rh * vsq / 6.0) - c->KC0 * UF;
                {
                    const double va[3] = {vx, vy, vz}, Fa[3] = {Fx, Fy, Fz};
                    for (int d = 0; d < 3; d++) {
                        const double eq1 = temp1 + c->K1 * rh * va[d] * va[d] * 0.5 + c->KC1 * (va[d] * Fa[d] - UF);
                        const double eq2 = va[d] * (c->K1 * rh + c->KC1 * Fa[d]);
                        gp[1 + 2 * d][id] = b * g[1 + 2 * d][id] + eq1 + eq2;
                        gp[2 + 2 * d][id] = b * g[2 + 2 * d][id] + eq1 - eq2;
                    }
                }
                {
                    const double temp2 = c->K2 * (3.0 * ph * mu + rh * (1.0 - vsq / 6.0));
                    /* pairs (7,8) x+y, (9,10) x-y, (11,12) x+z, (13,14) x-z, (15,16) y+z, (17,18) y-z */
                    const double wv[6] = {vx + vy, vx - vy, vx + vz, vx - vz, vy + vz, vy - vz};
                    const double wF[6] = {Fx + Fy, Fx - Fy, Fx + Fz, Fx - Fz, Fy + Fz, Fy - Fz};
                    for (int p = 0; p < 6; p++) {
                        const double eq1 = temp2 + c->K2 * rh * wv[p] * 0.5 * wv[p] + c->KC2 * (wv[p] * wF[p] - UF);
                        const double eq2 = c->K2 * rh * wv[p] + c->KC2 * wF[p];
                        gp[7 + 2 * p][id] = b * g[7 + 2 * p][id] + eq1 + eq2;
                        gp[8 + 2 * p][id] = b * g[8 + 2 * p][id] + eq1 - eq2;
                    }
                }
            }
        }
    }
}

/* D3Q7 and D3Q19 lattice vectors in the reference order
 * (src/stream_f.cu:52-59, src/stream_g.cu:56-76). */
static const int CF[7][3] = {{0, 0, 0}, {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
static const int CG[19][3] = {{0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},  {0, 0, -1},
                              {1, 1, 0},  {-1, -1, 0}, {1, -1, 0}, {-1, 1, 0}, {1, 0, 1},  {-1, 0, -1}, {1, 0, -1},
                              {-1, 0, 1}, {0, 1, 1},  {0, -1, -1}, {0, 1, -1}, {0, -1, 1}};

/* stream_f (src/stream_f.cu:52-59): ZSC eta-interpolated push,
 * f_i(x + c_i) = eta * P_i(x) + (1 - eta) * P_i(x + c_i), f_0(x) = P_0(x).
 * stream_g (src/stream_g.cu:56-76): g_i(x + c_i) = P_i(x).
 * Periodic wrap replaces the ghost exchanges (src/pack_mpi_f.cu, src/pack_mpi.cu
 * and their unpack twins with one rank). */
static void zo_stream(zo_ctx *s)
{
    const double eta = s->c.eta, eta2 = s->c.eta2;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < s->nz; z++) {
        for (int y = 0; y < s->ny; y++) {
            for (int x = 0; x < s->nx; x++) {
                const long id = zo_idx(s, x, y, z);
                s->f[0][id] = s->fp[0][id];
                for (int i = 1; i < 7; i++) {
                    const long d = zo_idx(s, wrap(x + CF[i][0], s->nx), wrap(y + CF[i][1], s->ny),
                                          wrap(z + CF[i][2], s->nz));
                    s->f[i][d] = eta * s->fp[i][id] + eta2 * s->fp[i][d];
                }
                s->g[0][id] = s->gp[0][id];
                for (int i = 1; i < 19; i++) {
                    const long d = zo_idx(s, wrap(x + CG[i][0], s->nx), wrap(y + CG[i][1], s->ny),
                                          wrap(z + CG[i][2], s->nz));
                    s->g[i][d] = s->gp[i][id];
                }
            }
        }
    }
}

/*
 * z-slabs: the same step split over ranks that each hold planes [z0, z0 + nz)
 * of a periodic box, as the reference splits it over MPI ranks
 * (src/vgrid.c:38-52), with its three halo exchanges per step
 * (src/main.cu:496-608): phi after update_phi (src/pack_mpi_phi.cu,
 * src/mpiupdate_phi.c), then the post-collision f and g before streaming
 * (src/pack_mpi_f.cu, src/pack_mpi.cu, src/mpiupdate*.c).  Here each exchange
 * moves whole planes: a rank sends its first plane to the rank below and its
 * last plane to the rank above, and receives the neighbours' planes as its
 * ghosts (side 0 below, side 1 above).  One step of a slab:
 *   zo_slab_moments; exchange phi (zo_slab_phi_plane -> zo_slab_set_phi_ghost);
 *   zo_slab_collide; exchange P, Q (zo_slab_post_plane -> zo_slab_set_post_ghost);
 *   zo_slab_stream.
 * Streaming pulls, f_i(x) = eta P_i(x - c_i) + (1 - eta) P_i(x) and
 * g_i(x) = Q_i(x - c_i) with the upstream values below / above the slab from
 * the ghosts: the same arithmetic as zo_stream's push, node for node.
 */
zo_ctx *zo_slab_create(int nx, int ny, int nz, const double *prm)
{
    if (nz < 1) return NULL;
    /* zo_create wants nz >= 3 for the periodic box; a slab may be thinner */
    zo_ctx *s = zo_create(nx, ny, nz < 3 ? 3 : nz, prm);
    if (!s) return NULL;
    s->nz = nz;
    s->n = (long)nx * ny * nz;
    s->slab = 1;
    const long nxy = (long)nx * ny;
    s->phi_ghost = (double *)calloc((size_t)(2 * nxy), sizeof(double));
    s->post_ghost = (double *)calloc((size_t)(2 * 26 * nxy), sizeof(double));
    if (!s->phi_ghost || !s->post_ghost) {
        zo_destroy(s);
        return NULL;
    }
    return s;
}

void zo_slab_moments(zo_ctx *s) { zo_moments_update(s); }

/* phi of the slab's first (side 0) or last (side 1) plane, nx*ny values */
void zo_slab_phi_plane(const zo_ctx *s, int side, double *out)
{
    const long nxy = (long)s->nx * s->ny;
    memcpy(out, s->phi + (side ? (long)(s->nz - 1) * nxy : 0), sizeof(double) * nxy);
}

/* the plane below (side 0) or above (side 1) the slab */
void zo_slab_set_phi_ghost(zo_ctx *s, int side, const double *in)
{
    const long nxy = (long)s->nx * s->ny;
    memcpy(s->phi_ghost + (side ? nxy : 0), in, sizeof(double) * nxy);
}

void zo_slab_collide(zo_ctx *s, double grav) { zo_collide(s, grav); }

/* post-collision P_0..P_6, Q_0..Q_18 of the first (side 0) or last (side 1)
 * plane: 26 x nx*ny values */
void zo_slab_post_plane(const zo_ctx *s, int side, double *out)
{
    const long nxy = (long)s->nx * s->ny, off = side ? (long)(s->nz - 1) * nxy : 0;
    for (int i = 0; i < 7; i++) memcpy(out + (long)i * nxy, s->fp[i] + off, sizeof(double) * nxy);
    for (int i = 0; i < 19; i++) memcpy(out + (long)(7 + i) * nxy, s->gp[i] + off, sizeof(double) * nxy);
}

void zo_slab_set_post_ghost(zo_ctx *s, int side, const double *in)
{
    const long nxy = (long)s->nx * s->ny;
    memcpy(s->post_ghost + (long)side * 26 * nxy, in, sizeof(double) * 26 * nxy);
}

/* post-collision field q (0..6 P, 7..25 Q) at (x, y, z) - c, z - c_z possibly
 * outside the slab (then from the ghost of that side) */
static inline double slab_upstream(const zo_ctx *s, int q, const double *arr, int x, int y, int z, const int *c)
{
    const long nxy = (long)s->nx * s->ny;
    const int xs = wrap(x - c[0], s->nx), ys = wrap(y - c[1], s->ny), zs = z - c[2];
    const long p = (long)xs + (long)s->nx * ys;
    if (zs < 0) return s->post_ghost[(long)q * nxy + p];
    if (zs >= s->nz) return s->post_ghost[(long)(26 + q) * nxy + p];
    return arr[zo_idx(s, xs, ys, zs)];
}

void zo_slab_stream(zo_ctx *s)
{
    const double eta = s->c.eta, eta2 = s->c.eta2;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < s->nz; z++) {
        for (int y = 0; y < s->ny; y++) {
            for (int x = 0; x < s->nx; x++) {
                const long id = zo_idx(s, x, y, z);
                s->f[0][id] = s->fp[0][id];
                for (int i = 1; i < 7; i++)
                    s->f[i][id] = eta * slab_upstream(s, i, s->fp[i], x, y, z, CF[i]) + eta2 * s->fp[i][id];
                s->g[0][id] = s->gp[0][id];
                for (int i = 1; i < 19; i++) s->g[i][id] = slab_upstream(s, 7 + i, s->gp[i], x, y, z, CG[i]);
            }
        }
    }
    s->steps++;
}

/* One or more steps in the order of src/main.cu:363-473 (relaxation loop) and
 * src/main.cu:496-608 (evolution loop); grav is grav_d (0 while relaxing). */
/*
 * Storage-rounding emulation (test aid for precision studies; no counterpart
 * in the reference, which stores FP32).  A GPU build that keeps the
 * post-collision sets in a 16-bit format stores, per node and population,
 *   f_0 as FP32, f_k (k = 1..6) as fmt(f_k * f_scale), g_i as
 *   fmt((g_i - shift_i) * g_scale),
 * the value formed in FP32 and rounded to nearest even.  zo_set_rounding
 * makes zo_step apply that round trip to the post-collision arrays, between
 * the collision and the streaming, with FP64 arithmetic everywhere else, so
 * that a run isolates the storage format's share of the error.
 * Formats: ZO_FMT_NONE, ZO_FMT_FP32, ZO_FMT_FP16 (IEEE binary16: 11
 * significant bits, subnormals below 2^-14, overflow above 65504), ZO_FMT_BF16
 * (8 significant bits, the FP32 exponent range).
 */
enum { ZO_FMT_NONE = 0, ZO_FMT_FP32 = 1, ZO_FMT_FP16 = 2, ZO_FMT_BF16 = 3 };

/* x rounded to nearest even with `bits` significant bits, the exponent of
 * its lowest bit at least `emin` (subnormals) */
static double round_sig(double x, int bits, int emin)
{
    if (x == 0.0 || !isfinite(x)) return x;
    int e;
    frexp(x, &e);                     /* |x| in [2^(e-1), 2^e) */
    int q = e - bits;                 /* exponent of the last kept bit */
    if (q < emin) q = emin;
    return ldexp(nearbyint(ldexp(x, -q)), q);
}

double zo_round(int fmt, double x)
{
    switch (fmt) {
    case ZO_FMT_FP32: return (double)(float)x;
    case ZO_FMT_FP16: {
        const double v = round_sig((double)(float)x, 11, -24);
        return fabs(v) > 65504.0 ? copysign(INFINITY, v) : v;
    }
    case ZO_FMT_BF16: return round_sig((double)(float)x, 8, -133);
    default: return x;
    }
}

void zo_round_array(int fmt, const double *in, double *out, long n)
{
    for (long i = 0; i < n; i++) out[i] = zo_round(fmt, in[i]);
}

void zo_set_rounding(zo_ctx *s, int f0_fmt, int f_fmt, double f_scale, int g_fmt, double g_scale,
                     const double *g_shift)
{
    s->round_f0 = f0_fmt;
    s->round_f = f_fmt;
    s->round_g = g_fmt;
    s->f_scale = f_scale;
    s->g_scale = g_scale;
    for (int i = 0; i < 19; i++) s->g_shift[i] = g_shift ? g_shift[i] : 0.0;
}

static void zo_round_post(zo_ctx *s)
{
    if (!s->round_f0 && !s->round_f && !s->round_g) return;
    const double fi = 1.0 / s->f_scale, gi = 1.0 / s->g_scale;
#pragma omp parallel for schedule(static)
    for (long id = 0; id < s->n; id++) {
        if (s->round_f0) s->fp[0][id] = zo_round(s->round_f0, s->fp[0][id]);
        if (s->round_f)
            for (int k = 1; k < 7; k++) s->fp[k][id] = zo_round(s->round_f, s->fp[k][id] * s->f_scale) * fi;
        if (s->round_g)
            for (int i = 0; i < 19; i++)
                s->gp[i][id] = zo_round(s->round_g, (s->gp[i][id] - s->g_shift[i]) * s->g_scale) * gi + s->g_shift[i];
    }
}

void zo_step(zo_ctx *s, int nsteps, double grav)
{
    for (int t = 0; t < nsteps; t++) {
        zo_moments_update(s);
        zo_collide(s, grav);
        zo_round_post(s);
        zo_stream(s);
        s->steps++;
    }
}

void zo_moments(const zo_ctx *s, double *phi, double *rho, double *ux, double *uy, double *uz)
{
    if (phi) memcpy(phi, s->phi, sizeof(double) * s->n);
    if (rho) memcpy(rho, s->rho, sizeof(double) * s->n);
    if (ux) memcpy(ux, s->ux, sizeof(double) * s->n);
    if (uy) memcpy(uy, s->uy, sizeof(double) * s->n);
    if (uz) memcpy(uz, s->uz, sizeof(double) * s->n);
}

/* Streamed distributions after the last step (reference lower halves). */
void zo_dist(const zo_ctx *s, double *f, double *g)
{
    for (int i = 0; i < 7; i++) if (f) memcpy(f + (long)i * s->n, s->f[i], sizeof(double) * s->n);
    for (int i = 0; i < 19; i++) if (g) memcpy(g + (long)i * s->n, s->g[i], sizeof(double) * s->n);
}

/*
 * Node-by-node comparison of a float32 state with the oracle's, without
 * copies: f (7 n), g (19 n) streamed distributions and mom (5 n: phi, rho,
 * ux, uy, uz), each NULL to skip.  out[2 q] = max |a - b| and out[2 q + 1] =
 * max |b| over field q, q = 0..6 f_0..f_6, 7..25 g_0..g_18, 26..30 the moments.
 * Non-finite differences count as infinite.
 */
void zo_compare(const zo_ctx *s, const float *f, const float *g, const float *mom, double *out)
{
    const long n = s->n;
    const double *ref[31];
    const float *got[31];
    for (int i = 0; i < 7; i++) { ref[i] = s->f[i]; got[i] = f ? f + (long)i * n : NULL; }
    for (int i = 0; i < 19; i++) { ref[7 + i] = s->g[i]; got[7 + i] = g ? g + (long)i * n : NULL; }
    const double *m[5] = {s->phi, s->rho, s->ux, s->uy, s->uz};
    for (int i = 0; i < 5; i++) { ref[26 + i] = m[i]; got[26 + i] = mom ? mom + (long)i * n : NULL; }
    for (int q = 0; q < 31; q++) {
        double dmax = 0.0, rmax = 0.0;
        if (got[q]) {
            const double *b = ref[q];
            const float *a = got[q];
#pragma omp parallel for reduction(max : dmax, rmax) schedule(static)
            for (long k = 0; k < n; k++) {
                double d = fabs((double)a[k] - b[k]);
                if (!(d == d) || d > 1e300) d = INFINITY;
                if (d > dmax) dmax = d;
                const double r = fabs(b[k]);
                if (r > rmax) rmax = r;
            }
        }
        out[2 * q] = dmax;
        out[2 * q + 1] = rmax;
    }
}

/* Overwrite the streamed distributions (resume from a snapshot). */
void zo_set_dist(zo_ctx *s, const double *f, const double *g)
{
    for (int i = 0; i < 7; i++) memcpy(s->f[i], f + (long)i * s->n, sizeof(double) * s->n);
    for (int i = 0; i < 19; i++) memcpy(s->g[i], g + (long)i * s->n, sizeof(double) * s->n);
}

/*
 * Statistics over the moment arrays.
 *  compat (reference region: x in [1, nx-2], y in [1, ny-2], all z;
 *  src/stats.c:39-55, src/logsave.c:63-147):
 *   out[0] umax = sqrt(max |u|^2)       out[1] vol = #(phi >= 0)
 *   out[2..4] mean u over phi >= 0      out[5] Ref = (0.75 vol / pi)^(1/3)
 *   out[6] Pin  out[7] Pout  out[8] Pin - Pout  out[9] Laplace error
 *   (src/logsave.c:135-162; Pout divides by nx*ny*nz - vol as the reference does)
 *  full domain:
 *   out[10] sum phi  out[11] sum rho  out[12..14] sum rho*u
 *   out[15] #(phi >= 0)  out[16] sqrt(max |u|^2)
 */
void zo_stats(const zo_ctx *s, double *out)
{
    const zo_const *c = &s->c;
    double umax2 = 0, vol = 0, sux = 0, suy = 0, suz = 0, pin = 0, pout = 0;
    double sphi = 0, srho = 0, mx = 0, my = 0, mz = 0, hv = 0, umax2f = 0;
#pragma omp parallel for schedule(static) reduction(max : umax2, umax2f) \
    reduction(+ : vol, sux, suy, suz, pin, pout, sphi, srho, mx, my, mz, hv)
    for (int z = 0; z < s->nz; z++) {
        for (int y = 0; y < s->ny; y++) {
            for (int x = 0; x < s->nx; x++) {
                const long id = zo_idx(s, x, y, z);
                const double ph = s->phi[id], rh = s->rho[id];
                const double u2 = s->ux[id] * s->ux[id] + s->uy[id] * s->uy[id] + s->uz[id] * s->uz[id];
                sphi += ph;
                srho += rh;
                mx += rh * s->ux[id];
                my += rh * s->uy[id];
                mz += rh * s->uz[id];
                if (ph >= 0.0) hv += 1.0;
                if (u2 > umax2f) umax2f = u2;
                if (x < 1 || x > s->nx - 2 || y < 1 || y > s->ny - 2) continue;
                if (u2 > umax2) umax2 = u2;
                double lap, gx, gy, gz;
                stencil(s, s->phi, NULL, x, y, z, &lap, &gx, &gy, &gz);
                const double ph2 = ph * ph;
                const double p = c->alpha * (ph2 * (3.0 * ph2 - 2.0 * c->phiStarSq) - c->phiStarSq * c->phiStarSq)
                                 - c->kappa * (ph * lap - 0.5 * (gx * gx + gy * gy + gz * gz)) + rh / 3.0;
                if (ph >= 0.0) {
                    vol += 1.0;
                    sux += s->ux[id];
                    suy += s->uy[id];
                    suz += s->uz[id];
                    pin += p;
                } else {
                    pout += p;
                }
            }
        }
    }
    const double volOut = (double)s->nx * s->ny * s->nz - vol;
    out[0] = sqrt(umax2);
    out[1] = vol;
    out[2] = vol > 0 ? sux / vol : 0.0;
    out[3] = vol > 0 ? suy / vol : 0.0;
    out[4] = vol > 0 ? suz / vol : 0.0;
    out[5] = pow(vol * 0.75 / M_PI, 1.0 / 3.0);
    out[6] = vol > 0 ? pin / vol : 0.0;
    out[7] = volOut > 0 ? pout / volOut : 0.0;
    out[8] = out[6] - out[7];
    out[9] = c->rc0 > 0.0 ? 0.5 * (2.0 * c->sigma / c->rc0 - out[8]) * c->rc0 / c->sigma : 0.0;
    out[10] = sphi;
    out[11] = srho;
    out[12] = mx;
    out[13] = my;
    out[14] = mz;
    out[15] = hv;
    out[16] = sqrt(umax2f);
}

int zo_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* Discrete adjoint (FP64).  No counterpart in the reference: it is the exact
 * transpose of the step restated above, used to check the GPU adjoint.
 *
 * Objectives on the moments of a streamed state (phi = sum f, rho = sum g,
 * u = sum c g / rho), with the smooth light-phase weight
 * w(phi) = (phiStar - phi) / (2 phiStar):
 *   0: mean over the last `window` states s^{T-window+1..T} of
 *      sum(w u_z) / sum(w)                         (light-phase rise velocity)
 *   1: sum(w z) / sum(w) of the final state s^T   (light-phase z-centroid,
 *      z = reference plane index = z + 1)
 * State s^k is the streamed (f, g) after k steps; s^0 the initial state.     */

static double zo_objective_state(const zo_ctx *s, const double *const *f, const double *const *g, int objective,
                                 double *A_out, double *B_out)
{
    const double phiStar = s->c.phiStar;
    double A = 0.0, B = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : A, B)
    for (long id = 0; id < s->n; id++) {
        double ph = 0.0, rh = 0.0;
        for (int i = 0; i < 7; i++) ph += f[i][id];
        for (int i = 0; i < 19; i++) rh += g[i][id];
        const double w = (phiStar - ph) / (2.0 * phiStar);
        if (objective == 0) {
            const double mz = g[5][id] - g[6][id] + g[11][id] - g[12][id] - g[13][id] + g[14][id] + g[15][id]
                              - g[16][id] - g[17][id] + g[18][id];
            A += w * mz / rh;
        } else {
            const long z = id / ((long)s->nx * s->ny);
            A += w * (double)(z + 1);
        }
        B += w;
    }
    *A_out = A;
    *B_out = B;
    return A / B;
}

/* Add d(scale * A/B)/d(state) to (lf, lg) at every node. */
static void zo_objective_source(const zo_ctx *s, const double *const *f, const double *const *g, int objective,
                                double scale, double A, double B, double **lf, double **lg)
{
    const double phiStar = s->c.phiStar;
    const double dw = -1.0 / (2.0 * phiStar);
    const double ratio = A / B;
#pragma omp parallel for schedule(static)
    for (long id = 0; id < s->n; id++) {
        double ph = 0.0, rh = 0.0;
        for (int i = 0; i < 7; i++) ph += f[i][id];
        for (int i = 0; i < 19; i++) rh += g[i][id];
        const double w = (phiStar - ph) / (2.0 * phiStar);
        double dphi, drho = 0.0, dmz = 0.0;
        if (objective == 0) {
            const double mz = g[5][id] - g[6][id] + g[11][id] - g[12][id] - g[13][id] + g[14][id] + g[15][id]
                              - g[16][id] - g[17][id] + g[18][id];
            const double uz = mz / rh;
            dphi = scale * dw * (uz - ratio) / B;
            const double duz = scale * w / B;
            dmz = duz / rh;
            drho = -duz * uz / rh;
        } else {
            const long z = id / ((long)s->nx * s->ny);
            dphi = scale * dw * ((double)(z + 1) - ratio) / B;
        }
        for (int i = 0; i < 7; i++) lf[i][id] += dphi;
        for (int i = 0; i < 19; i++) lg[i][id] += drho + (double)CG[i][2] * dmz;
    }
}

/* One adjoint step.  In: the streamed state s^n (f, g), lambda^{n+1}
 * (lf_in, lg_in).  Out: lambda^n (lf_out, lg_out), without objective sources;
 * dgrav += sum over nodes of lambda_{F_z} H(phi > 0). */
static void zo_adjoint_step(const zo_ctx *s, const double *const *f, const double *const *g, const double *const *lf_in,
                            const double *const *lg_in, double grav, double **lf_out, double **lg_out, double *dgrav,
                            double *phi, double *llap, double *lgx, double *lgy, double *lgz)
{
    const zo_const *c = &s->c;
    (void)grav;
#pragma omp parallel for schedule(static)
    for (long id = 0; id < s->n; id++) {
        double ph = 0.0;
        for (int i = 0; i < 7; i++) ph += f[i][id];
        phi[id] = ph;
    }
    double dg = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : dg)
    for (int z = 0; z < s->nz; z++) {
        for (int y = 0; y < s->ny; y++) {
            for (int x = 0; x < s->nx; x++) {
                const long id = zo_idx(s, x, y, z);
                /* forward quantities at the node */
                double lap, gr[3];
                stencil(s, phi, NULL, x, y, z, &lap, &gr[0], &gr[1], &gr[2]);
                const double ph = phi[id];
                double rh = 0.0, m[3] = {0, 0, 0};
                for (int i = 0; i < 19; i++) {
                    rh += g[i][id];
                    for (int k = 0; k < 3; k++) m[k] += CG[i][k] * g[i][id];
                }
                const double u[3] = {m[0] / rh, m[1] / rh, m[2] / rh};
                const double mu = c->alpha4 * ph * (ph * ph - c->phiStarSq) - c->kappa * lap;
                double F[3] = {mu * gr[0], mu * gr[1], mu * gr[2]};
                const int heavy = ph > 0.0;
                if (heavy) F[2] += grav;
                const double us[3] = {u[0] + 0.5 * F[0] / rh, u[1] + 0.5 * F[1] / rh, u[2] + 0.5 * F[2] / rh};
                const double v[3] = {3.0 * us[0], 3.0 * us[1], 3.0 * us[2]};
                const double vsq6 = (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / 6.0;
                const double Cf = c->invTauPhi * c->invEta2 * ph;

                /* stream adjoint: lambda of the post-collision values at this node */
                double lP[7], lQ[19];
                lP[0] = lf_in[0][id];
                for (int i = 1; i < 7; i++) {
                    const long dn = zo_idx(s, wrap(x + CF[i][0], s->nx), wrap(y + CF[i][1], s->ny),
                                           wrap(z + CF[i][2], s->nz));
                    lP[i] = c->eta * lf_in[i][dn] + c->eta2 * lf_in[i][id];
                }
                for (int i = 0; i < 19; i++) {
                    const long dn = zo_idx(s, wrap(x + CG[i][0], s->nx), wrap(y + CG[i][1], s->ny),
                                           wrap(z + CG[i][2], s->nz));
                    lQ[i] = lg_in[i][dn];
                }

                /* D3Q7 collision */
                double lphi = 0.0, lmu = 0.0, lus[3] = {0, 0, 0}, lF[3] = {0, 0, 0}, lrho = 0.0;
                {
                    const double lAf = -6.0 * lP[0] + lP[1] + lP[2] + lP[3] + lP[4] + lP[5] + lP[6];
                    double lCf = 0.0;
                    for (int k = 0; k < 3; k++) {
                        const double d = lP[1 + 2 * k] - lP[2 + 2 * k];
                        lCf += us[k] * d;
                        lus[k] += Cf * d;
                    }
                    lphi += c->invTauPhi * lP[0] + c->invTauPhi * c->invEta2 * lCf;
                    lmu += 0.5 * c->Gamma * c->invTauPhi * lAf;
                }
                /* D3Q19 collision with forcing */
                double ls = 0.0, lvsq6 = 0.0, lUF = 0.0, lv[3] = {0, 0, 0};
                {
                    ls += -2.0 * c->K0 * lQ[0];
                    lrho += c->K0 * (1.0 - vsq6) * lQ[0];
                    lvsq6 += -c->K0 * rh * lQ[0];
                    lUF += -c->KC0 * lQ[0];
                    double ltemp1 = 0.0;
                    for (int k = 0; k < 3; k++) {
                        const double S = lQ[1 + 2 * k] + lQ[2 + 2 * k], A = lQ[1 + 2 * k] - lQ[2 + 2 * k];
                        ltemp1 += S;
                        lrho += 0.5 * c->K1 * v[k] * v[k] * S + c->K1 * v[k] * A;
                        lv[k] += c->K1 * rh * v[k] * S + c->KC1 * F[k] * S + (c->K1 * rh + c->KC1 * F[k]) * A;
                        lF[k] += c->KC1 * v[k] * S + c->KC1 * v[k] * A;
                        lUF += -c->KC1 * S;
                    }
                    ls += c->K1 * ltemp1;
                    lrho += c->K1 * (1.0 - vsq6) * ltemp1;
                    lvsq6 += -c->K1 * rh * ltemp1;
                    /* pairs (7,8) x+y, (9,10) x-y, (11,12) x+z, (13,14) x-z, (15,16) y+z, (17,18) y-z */
                    static const int PA[6] = {0, 0, 0, 0, 1, 1}, PB[6] = {1, 1, 2, 2, 2, 2};
                    static const double SG[6] = {1, -1, 1, -1, 1, -1};
                    double ltemp2 = 0.0;
                    for (int p = 0; p < 6; p++) {
                        const int a = PA[p], b = PB[p];
                        const double sg = SG[p];
                        const double w = v[a] + sg * v[b], G = F[a] + sg * F[b];
                        const double S = lQ[7 + 2 * p] + lQ[8 + 2 * p], A = lQ[7 + 2 * p] - lQ[8 + 2 * p];
                        ltemp2 += S;
                        lrho += 0.5 * c->K2 * w * w * S + c->K2 * w * A;
                        const double lw = c->K2 * rh * w * S + c->KC2 * G * S + c->K2 * rh * A;
                        const double lG = c->KC2 * w * S + c->KC2 * A;
                        lUF += -c->KC2 * S;
                        lv[a] += lw;
                        lv[b] += sg * lw;
                        lF[a] += lG;
                        lF[b] += sg * lG;
                    }
                    ls += c->K2 * ltemp2;
                    lrho += c->K2 * (1.0 - vsq6) * ltemp2;
                    lvsq6 += -c->K2 * rh * ltemp2;
                }
                for (int k = 0; k < 3; k++) lv[k] += lvsq6 * v[k] / 3.0;
                for (int k = 0; k < 3; k++) {
                    lus[k] += lUF * F[k] + 3.0 * lv[k];
                    lF[k] += lUF * us[k];
                }
                lphi += 3.0 * mu * ls;
                lmu += 3.0 * ph * ls;
                /* us = u + 0.5 F / rho, u = m / rho */
                double lm[3];
                for (int k = 0; k < 3; k++) {
                    lF[k] += 0.5 * lus[k] / rh;
                    lrho += -0.5 * lus[k] * F[k] / (rh * rh);
                    lm[k] = lus[k] / rh;
                    lrho += -lus[k] * u[k] / rh;
                }
                /* F = mu grad (+ grav on phi > 0) */
                for (int k = 0; k < 3; k++) lmu += gr[k] * lF[k];
                if (heavy) dg += lF[2];
                lgx[id] = mu * lF[0];
                lgy[id] = mu * lF[1];
                lgz[id] = mu * lF[2];
                /* mu = alpha4 phi (phi^2 - phiStar^2) - kappa lap */
                lphi += c->alpha4 * (3.0 * ph * ph - c->phiStarSq) * lmu;
                llap[id] = -c->kappa * lmu;
                /* collisions' direct terms and the moments */
                lf_out[0][id] = c->invTauPhiOne * lP[0] + lphi;
                for (int i = 1; i < 7; i++) lf_out[i][id] = c->invTauPhiOne * lP[i] + lphi;
                for (int i = 0; i < 19; i++)
                    lg_out[i][id] = c->invTauRhoOne * lQ[i] + lrho + CG[i][0] * lm[0] + CG[i][1] * lm[1]
                                    + CG[i][2] * lm[2];
            }
        }
    }
    *dgrav += dg;
    /* transposed stencils: lapT = lap (symmetric), gradT = -grad (antisymmetric) */
#pragma omp parallel for schedule(static)
    for (int z = 0; z < s->nz; z++) {
        for (int y = 0; y < s->ny; y++) {
            for (int x = 0; x < s->nx; x++) {
                const long id = zo_idx(s, x, y, z);
                double l1, d, gxv, gyv, gzv;
                stencil(s, llap, NULL, x, y, z, &l1, &d, &d, &d);
                stencil(s, lgx, NULL, x, y, z, &d, &gxv, &d, &d);
                stencil(s, lgy, NULL, x, y, z, &d, &d, &gyv, &d);
                stencil(s, lgz, NULL, x, y, z, &d, &d, &d, &gzv);
                const double add = l1 - gxv - gyv - gzv;
                for (int i = 0; i < 7; i++) lf_out[i][id] += add;
            }
        }
    }
}

/* J and its adjoint over T steps from the current state s^0, storing every
 * state (test sizes).  dgrav receives dJ/dgrav; lf0 (7N) / lg0 (19N) receive
 * dJ/ds^0.  The context ends at s^T. */
double zo_adjoint_run(zo_ctx *s, int T, double grav, int objective, int window, double *dgrav, double *lf0,
                      double *lg0)
{
    const long N = s->n;
    double *store = (double *)malloc(sizeof(double) * 26 * N * (size_t)(T + 1));
    double *work = (double *)calloc((size_t)(26 * 2 + 5) * N, sizeof(double));
    if (!store || !work) {
        free(store);
        free(work);
        return NAN;
    }
    for (int i = 0; i < 7; i++) memcpy(store + (long)i * N, s->f[i], sizeof(double) * N);
    for (int i = 0; i < 19; i++) memcpy(store + (long)(7 + i) * N, s->g[i], sizeof(double) * N);
    for (int k = 1; k <= T; k++) {
        zo_step(s, 1, grav);
        double *st = store + (size_t)k * 26 * N;
        for (int i = 0; i < 7; i++) memcpy(st + (long)i * N, s->f[i], sizeof(double) * N);
        for (int i = 0; i < 19; i++) memcpy(st + (long)(7 + i) * N, s->g[i], sizeof(double) * N);
    }
    double *la[26], *lb[26];
    for (int i = 0; i < 26; i++) {
        la[i] = work + (long)i * N;
        lb[i] = work + (long)(26 + i) * N;
    }
    double *phi = work + 52L * N, *llap = work + 53L * N, *lgx = work + 54L * N, *lgy = work + 55L * N,
           *lgz = work + 56L * N;
    const double *fk[7], *gk[19];
    double J = 0.0, A, B;
    const int first = objective == 0 ? T - window + 1 : T;
    const double scale = objective == 0 ? 1.0 / window : 1.0;
    /* lambda^T: source of the final state */
    {
        double *st = store + (size_t)T * 26 * N;
        for (int i = 0; i < 7; i++) fk[i] = st + (long)i * N;
        for (int i = 0; i < 19; i++) gk[i] = st + (long)(7 + i) * N;
        J += scale * zo_objective_state(s, fk, gk, objective, &A, &B);
        zo_objective_source(s, fk, gk, objective, scale, A, B, la, la + 7);
    }
    *dgrav = 0.0;
    for (int k = T - 1; k >= 0; k--) {
        double *st = store + (size_t)k * 26 * N;
        for (int i = 0; i < 7; i++) fk[i] = st + (long)i * N;
        for (int i = 0; i < 19; i++) gk[i] = st + (long)(7 + i) * N;
        zo_adjoint_step(s, fk, gk, (const double *const *)la, (const double *const *)(la + 7), grav, lb, lb + 7,
                        dgrav, phi, llap, lgx, lgy, lgz);
        if (k >= first) {
            J += scale * zo_objective_state(s, fk, gk, objective, &A, &B);
            zo_objective_source(s, fk, gk, objective, scale, A, B, lb, lb + 7);
        }
        for (int i = 0; i < 26; i++) {
            double *t = la[i];
            la[i] = lb[i];
            lb[i] = t;
        }
    }
    for (int i = 0; i < 7; i++) memcpy(lf0 + (long)i * N, la[i], sizeof(double) * N);
    for (int i = 0; i < 19; i++) memcpy(lg0 + (long)i * N, la[7 + i], sizeof(double) * N);
    free(store);
    free(work);
    return J;
}

/* J alone (forward only), for finite differences. */
double zo_objective_run(zo_ctx *s, int T, double grav, int objective, int window)
{
    const int first = objective == 0 ? T - window + 1 : T;
    const double scale = objective == 0 ? 1.0 / window : 1.0;
    double J = 0.0, A, B;
    const double *fk[7], *gk[19];
    for (int k = 0; k <= T; k++) {
        if (k > 0) zo_step(s, 1, grav);
        if (k >= first) {
            for (int i = 0; i < 7; i++) fk[i] = s->f[i];
            for (int i = 0; i < 19; i++) gk[i] = s->g[i];
            J += scale * zo_objective_state(s, fk, gk, objective, &A, &B);
        }
    }
    return J;
}

/* dJ/dphi0 and dJ/drho0 from dJ/ds^0 through the initial equilibrium
 * (src/init_f.cu:57-78, src/init_g.cu:69-91) with periodic z. */
void zo_init_adjoint(const zo_ctx *s, const double *phi0, const double *lf0, const double *lg0, double *lphi0,
                     double *lrho0)
{
    const zo_const *c = &s->c;
    const long N = s->n;
    double *llap = (double *)malloc(sizeof(double) * N);
#pragma omp parallel for schedule(static)
    for (int z = 0; z < s->nz; z++) {
        for (int y = 0; y < s->ny; y++) {
            for (int x = 0; x < s->nx; x++) {
                const long id = zo_idx(s, x, y, z);
                double lap, gx, gy, gz;
                stencil(s, phi0, NULL, x, y, z, &lap, &gx, &gy, &gz);
                const double ph = phi0[id];
                const double mu = c->alpha4 * ph * (ph * ph - c->phiStarSq) - c->kappa * lap;
                const double l0 = lf0[id];
                double lfs = 0.0, lga = 0.0, lgd = 0.0;
                for (int i = 1; i < 7; i++) lfs += lf0[i * N + id];
                for (int i = 1; i < 7; i++) lga += lg0[i * N + id];
                for (int i = 7; i < 19; i++) lgd += lg0[i * N + id];
                const double lg00 = lg0[id];
                /* f0 = phi - 3 Gamma mu; fi = Gamma mu / 2; g0 = W0 (rho - 6 phi mu);
                 * g axis = W1 (3 phi mu + rho); g diag = W2 (3 phi mu + rho) */
                const double lmu = -3.0 * c->Gamma * l0 + 0.5 * c->Gamma * lfs - 6.0 * ZO_W0 * ph * lg00
                                   + 3.0 * ZO_W1 * ph * lga + 3.0 * ZO_W2 * ph * lgd;
                double lphi = l0 - 6.0 * ZO_W0 * mu * lg00 + 3.0 * ZO_W1 * mu * lga + 3.0 * ZO_W2 * mu * lgd;
                lphi += c->alpha4 * (3.0 * ph * ph - c->phiStarSq) * lmu;
                llap[id] = -c->kappa * lmu;
                lphi0[id] = lphi;
                if (lrho0) lrho0[id] = ZO_W0 * lg00 + ZO_W1 * lga + ZO_W2 * lgd;
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (int z = 0; z < s->nz; z++) {
        for (int y = 0; y < s->ny; y++) {
            for (int x = 0; x < s->nx; x++) {
                double l1, d;
                stencil(s, llap, NULL, x, y, z, &l1, &d, &d, &d);
                lphi0[zo_idx(s, x, y, z)] += l1;
            }
        }
    }
    free(llap);
}

/* Heavy-node log for finite-difference checks of the adjoint.  The gravity
 * term is switched on by H(phi > 0) (src/collision_f.cu:96), so J is only
 * piecewise smooth in the force: nodes whose phi crosses zero make finite
 * differences jump.  mode 1 records H of every node and collision for `steps`
 * collisions after the next zo_init; mode 2 replays the recorded H instead of
 * testing phi (the forward map with the heavy set frozen, whose derivative is
 * what the discrete adjoint computes); mode 0 frees the log.  Returns 0, or
 * -1 when the log cannot be allocated or replay has nothing recorded. */
int zo_heavy_mask(zo_ctx *s, int mode, long steps)
{
    s->heavy_pos = 0;
    if (mode == 0) {
        free(s->heavy_log);
        s->heavy_log = NULL;
        s->heavy_cap = 0;
        s->heavy_mode = 0;
        return 0;
    }
    if (mode == 1) {
        free(s->heavy_log);
        s->heavy_cap = steps * s->n;
        s->heavy_log = (unsigned char *)malloc((size_t)s->heavy_cap);
        if (!s->heavy_log) {
            s->heavy_cap = 0;
            s->heavy_mode = 0;
            return -1;
        }
        s->heavy_mode = 1;
        return 0;
    }
    if (mode == 2 && s->heavy_log) {
        s->heavy_mode = 2;
        return 0;
    }
    return -1;
}

/* One adjoint step at the current streamed state s^n: (lf_out, lg_out) =
 * J^T (lf_in, lg_in), J the derivative of the step s^n -> s^{n+1}
 * (zo_adjoint_step, no objective source); *dgrav receives
 * sum lambda_{F_z} H(phi > 0).  Test aid for the per-step dot-product check
 * <J v, w> = <v, J^T w>.  Arrays: 7 x N (f) and 19 x N (g).  Returns 0, or
 * -1 when the scratch cannot be allocated. */
int zo_adjoint_apply(zo_ctx *s, double grav, const double *lf_in, const double *lg_in, double *lf_out,
                     double *lg_out, double *dgrav)
{
    const long N = s->n;
    double *work = (double *)calloc((size_t)5 * N, sizeof(double));
    if (!work) return -1;
    const double *fk[7], *gk[19], *la[26];
    double *lb[26];
    for (int i = 0; i < 7; i++) {
        fk[i] = s->f[i];
        la[i] = lf_in + (long)i * N;
        lb[i] = lf_out + (long)i * N;
    }
    for (int i = 0; i < 19; i++) {
        gk[i] = s->g[i];
        la[7 + i] = lg_in + (long)i * N;
        lb[7 + i] = lg_out + (long)i * N;
    }
    *dgrav = 0.0;
    zo_adjoint_step(s, fk, gk, (const double *const *)la, (const double *const *)(la + 7), grav, lb, lb + 7, dgrav,
                    work, work + N, work + 2 * N, work + 3 * N, work + 4 * N);
    free(work);
    return 0;
}
