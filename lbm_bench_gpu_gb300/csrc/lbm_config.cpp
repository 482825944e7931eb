// lbm_config.cpp -- input files and derived constants (host only).
//
// lbm_read_inputs follows src/paramread.c:36-75: both files are read as a
// stream of whitespace-separated tokens; header tokens are skipped by count
// and values are converted with the same scanf conversions (%d, %f).
// lbm::derive follows src/paramread.c:141-170 (evaluated in double, stored as
// float).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "lbm_internal.h"

namespace lbm {

namespace {
thread_local std::string g_last_error;

constexpr double kW0 = 1.0 / 3.0, kW1 = 1.0 / 18.0, kW2 = 1.0 / 36.0;  // src/constants.h:52-54
constexpr double kWC0 = 1.0, kWC1 = 1.0 / 6.0, kWC2 = 1.0 / 12.0;       // src/constants.h:57-59

struct File {
    FILE *fp;
    explicit File(const std::string &path) : fp(std::fopen(path.c_str(), "r")) {}
    ~File()
    {
        if (fp) std::fclose(fp);
    }
    bool skip(int ntokens)
    {
        char tmp[256];
        for (int i = 0; i < ntokens; i++)
            if (std::fscanf(fp, "%255s", tmp) != 1) return false;
        return true;
    }
    bool ints(int n, int *const *dst)
    {
        for (int i = 0; i < n; i++)
            if (std::fscanf(fp, "%d", dst[i]) != 1) return false;
        return true;
    }
    bool floats(int n, float *const *dst)
    {
        for (int i = 0; i < n; i++)
            if (std::fscanf(fp, "%f", dst[i]) != 1) return false;
        return true;
    }
};

std::string join(const char *dir, const char *name)
{
    if (!dir || !*dir) return name;
    std::string s(dir);
    if (s.back() != '/') s += '/';
    return s + name;
}
}  // namespace

void set_error(const std::string &msg) { g_last_error = msg; }
const std::string &last_error() { return g_last_error; }

void derive(const lbm_params &p, lbm_derived &d)
{
    const double rhoL = p.rhoL, rhoH = p.rhoH, tauRho = p.tauRho, tauPhi = p.tauPhi;
    const double width = p.width, sigma = p.sigma, Eo = p.Eo, rc0 = p.rc0;
    const double phiStar = 0.5 * (rhoH - rhoL);
    const double phiStarSq = phiStar * phiStar;
    const double invTauRho = 1.0 / tauRho;
    const double invTauRhoHalf = 1.0 - 0.5 * invTauRho;
    const double eta = 1.0 / (tauPhi + 0.5);
    const double alpha = 0.75 * sigma / (width * phiStarSq * phiStarSq);
    const double kappa = (width * phiStar) * (width * phiStar) * alpha * 0.5;
    const double gravity = 0.25 * Eo * sigma / ((rhoH - rhoL) * rc0 * rc0);
    d.phiStar = (float)phiStar;
    d.phiStarSq = (float)phiStarSq;
    d.invTauRho = (float)invTauRho;
    d.invTauRhoOne = (float)(1.0 - invTauRho);
    d.invTauRhoHalf = (float)invTauRhoHalf;
    d.eta = (float)eta;
    d.eta2 = (float)(1.0 - eta);
    d.invEta2 = (float)(0.5 / (1.0 - eta));
    d.invTauPhi = (float)(1.0 / tauPhi);
    d.invTauPhiOne = (float)(1.0 - 1.0 / tauPhi);
    d.alpha = (float)alpha;
    d.alpha4 = (float)(4.0 * alpha);
    d.kappa = (float)kappa;
    d.gravity = (float)gravity;
    d.grav = (float)(2.0 * phiStar * gravity);
    d.K0 = (float)(invTauRho * kW0);
    d.K1 = (float)(invTauRho * kW1);
    d.K2 = (float)(invTauRho * kW2);
    d.KC0 = (float)(invTauRhoHalf * kWC0);
    d.KC1 = (float)(invTauRhoHalf * kWC1);
    d.KC2 = (float)(invTauRhoHalf * kWC2);
}

StepConst step_const(const lbm_derived &d, const lbm_params &p, float grav)
{
    StepConst c;
    c.eta = d.eta;
    c.eta2 = d.eta2;
    c.alpha4 = d.alpha4;
    c.kappa = d.kappa;
    c.phiStarSq = d.phiStarSq;
    c.Gamma = p.Gamma;
    c.invTauPhi = d.invTauPhi;
    c.invTauPhiOne = d.invTauPhiOne;
    c.invEta2 = d.invEta2;
    c.invTauRhoOne = d.invTauRhoOne;
    c.K0 = d.K0;
    c.K1 = d.K1;
    c.K2 = d.K2;
    c.KC0 = d.KC0;
    c.KC1 = d.KC1;
    c.KC2 = d.KC2;
    c.grav = grav;
    return c;
}

}  // namespace lbm

extern "C" int lbm_read_inputs(const char *dir, lbm_params *p, lbm_run *run, float *bubbles, int max_bubbles,
                               int *nbubbles)
{
    if (!p) {
        lbm::set_error("lbm_read_inputs: p is NULL");
        return LBM_EINVAL;
    }
    lbm_params q;
    std::memset(&q, 0, sizeof(q));
    lbm_run r;
    std::memset(&r, 0, sizeof(r));
    {
        const std::string path = lbm::join(dir, "properties.in");
        lbm::File f(path);
        if (!f.fp) {
            lbm::set_error("cannot open " + path);
            return LBM_EIO;
        }
        int *i4[] = {&r.max_step, &r.relax_step, &r.save, &r.stat};
        int *i3[] = {&q.nx, &q.ny, &q.nz};
        int *i2[] = {&q.block_x, &q.block_y};
        float *rho[] = {&q.rhoL, &q.rhoH};
        float *tau[] = {&q.tauRho, &q.tauPhi};
        float *wsg[] = {&q.width, &q.sigma, &q.Gamma};
        float *eo[] = {&q.Eo};
        const bool ok = f.skip(4) && f.ints(4, i4) && f.skip(3) && f.ints(3, i3) && f.skip(2) && f.ints(2, i2)
                        && f.skip(2) && f.floats(2, rho) && f.skip(2) && f.floats(2, tau) && f.skip(3)
                        && f.floats(3, wsg) && f.skip(1) && f.floats(1, eo);
        if (!ok) {
            lbm::set_error("malformed " + path);
            return LBM_EIO;
        }
    }
    int nb = 0;
    {
        const std::string path = lbm::join(dir, "discrete.in");
        lbm::File f(path);
        if (!f.fp) {
            lbm::set_error("cannot open " + path);
            return LBM_EIO;
        }
        int *n1[] = {&nb};
        if (!(f.skip(1) && f.ints(1, n1) && f.skip(4)) || nb < 0) {
            lbm::set_error("malformed " + path);
            return LBM_EIO;
        }
        for (int m = 0; m < nb; m++) {
            float v[4];
            float *pv[] = {&v[0], &v[1], &v[2], &v[3]};
            if (!f.floats(4, pv)) {
                lbm::set_error("malformed " + path + ": fewer bubble rows than announced");
                return LBM_EIO;
            }
            if (m == 0) q.rc0 = v[3];
            if (bubbles && m < max_bubbles) std::memcpy(bubbles + 4 * m, v, sizeof(v));
        }
    }
    q.storage = LBM_STORAGE_FP32;
    q.device = 0;
    q.compat = 1;
    *p = q;
    if (run) *run = r;
    if (nbubbles) *nbubbles = nb;
    return LBM_OK;
}

namespace lbm {
// The physical parameters every entry point needs before it derives the
// constants (src/paramread.c:141-170 divides by tauRho, tauPhi, width and
// rhoH - rhoL, and by rc0 when Eo is not zero); nullptr when they are usable.
const char *physics_error(const lbm_params &p)
{
    if (!(p.tauRho > 0.f) || !(p.tauPhi > 0.f) || !(p.width > 0.f))
        return "tauRho, tauPhi and width must be positive";
    if (!(p.rhoH != p.rhoL)) return "rhoH must differ from rhoL";
    if (p.Eo != 0.f && !(p.rc0 > 0.f)) return "rc0 must be positive when Eo is not zero";
    return nullptr;
}
}  // namespace lbm

extern "C" int lbm_derive(const lbm_params *p, lbm_derived *d)
{
    if (!p || !d) {
        lbm::set_error("lbm_derive: NULL argument");
        return LBM_EINVAL;
    }
    lbm::derive(*p, *d);
    return LBM_OK;
}

extern "C" const char *lbm_strerror(int code)
{
    switch (code) {
    case LBM_OK: return "ok";
    case LBM_EINVAL: return "invalid argument";
    case LBM_ENOMEM: return "out of memory";
    case LBM_ECUDA: return "CUDA error";
    case LBM_ENAN: return "non-finite values in the state";
    case LBM_ETIMEOUT: return "device wait timed out";
    case LBM_EIO: return "input file missing or malformed";
    case LBM_ESTATE: return "call out of order";
    default: return "unknown status";
    }
}

extern "C" const char *lbm_last_error(void) { return lbm::last_error().c_str(); }
