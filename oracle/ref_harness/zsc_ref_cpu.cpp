/*
 * zsc_ref_cpu.cpp -- runs the reference's own step kernels on the host CPU.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build.py compiles this file together
 * with the unmodified reference sources (included below by name, found through
 * -I on the reference's src/ directory) into oracle/_ref/libzsc_ref.so.  It is
 * used to pin the FP64 oracle (golden vectors) and as the CPU arm of bench.py
 * (--impl reference).  Nothing in the product links it.
 *
 * The launch sequence is the one of the reference driver: setup as in
 * src/main.cu:155-357 and one loop iteration as in src/main.cu:496-608
 * (update_phi, update_rho, update_velocity, phi halo, collision_f,
 * collision_g, f halo, stream_f, stream_g, distribution halo).  Kernels are
 * launched by a CPU emulation of the CUDA grid: blocks are spread over OpenMP
 * threads (every kernel of the step writes each output element from exactly
 * one thread, so this is race-free); threads of a block run in order.
 */
#include "ref_shim.h"
#include <unistd.h>
#ifdef _OPENMP
#include <omp.h>
#endif

thread_local zr_dim3 blockIdx, threadIdx, blockDim;
void *zr_mpi_recv_buf[8];

/* The reference sources, in the order src/main.cu includes them (the VTK
 * writer is left out: it is output only). */
#include "constants.h"
#include "gridid.c"
#include "init.c"
#include "paramread.c"
#include "logsave.c"
#include "stats.c"
#include "mpiupdate.c"
#include "mpiupdate_f.c"
#include "mpiupdate_phi.c"
#include "vgrid.c"
#include "init_f.cu"
#include "init_g.cu"
#include "update_phi.cu"
#include "update_rho.cu"
#include "update_velocity.cu"
#include "collision_f.cu"
#include "collision_g.cu"
#include "pack_mpi.cu"
#include "pack_mpi_f.cu"
#include "pack_mpi_phi.cu"
#include "stream_f.cu"
#include "stream_g.cu"
#include "unpack_mpi.cu"
#include "unpack_mpi_f.cu"
#include "unpack_mpi_phi.cu"

namespace {

zr_dim3 grid_dim, block_dim;

int *nb_e, *nb_w, *nb_n, *nb_s;             /* host neighbour tables */
float *phi_h, *rho_h, *ux_h, *uy_h, *uz_h;  /* host fields */
int *nb_e_d, *nb_w_d, *nb_n_d, *nb_s_d;     /* "device" copies */
float *phi_d, *rho_d, *ux_d, *uy_d, *uz_d;
float *f_d[7], *g_d[19];
float *top_snd_d, *bot_snd_d, *top_rcv_d, *bot_rcv_d;
float *topF_snd_d, *botF_snd_d, *topF_rcv_d, *botF_rcv_d;
float *top_snd_h, *bot_snd_h, *top_rcv_h, *bot_rcv_h;
float *topF_snd_h, *botF_snd_h, *topF_rcv_h, *botF_rcv_h;
bool ready = false;

template <typename K>
void launch(K &&kernel)
{
#pragma omp parallel for collapse(2) schedule(static)
    for (int by = 0; by < grid_dim.y; by++) {
        for (int bx = 0; bx < grid_dim.x; bx++) {
            blockIdx = zr_dim3{bx, by, 0};
            blockDim = block_dim;
            for (int ty = 0; ty < block_dim.y; ty++) {
                for (int tx = 0; tx < block_dim.x; tx++) {
                    threadIdx = zr_dim3{tx, ty, 0};
                    kernel();
                }
            }
        }
    }
}

void release()
{
    void *ptrs[] = {nb_e, nb_w, nb_n, nb_s, phi_h, rho_h, ux_h, uy_h, uz_h,
                    nb_e_d, nb_w_d, nb_n_d, nb_s_d, phi_d, rho_d, ux_d, uy_d, uz_d,
                    top_snd_d, bot_snd_d, top_rcv_d, bot_rcv_d, topF_snd_d, botF_snd_d, topF_rcv_d, botF_rcv_d,
                    top_snd_h, bot_snd_h, top_rcv_h, bot_rcv_h, topF_snd_h, botF_snd_h, topF_rcv_h, botF_rcv_h};
    for (void *p : ptrs) free(p);
    for (int i = 0; i < 7; i++) { free(f_d[i]); f_d[i] = nullptr; }
    for (int i = 0; i < 19; i++) { free(g_d[i]); g_d[i] = nullptr; }
    nb_e = nb_w = nb_n = nb_s = nullptr;
    phi_h = rho_h = ux_h = uy_h = uz_h = nullptr;
    nb_e_d = nb_w_d = nb_n_d = nb_s_d = nullptr;
    phi_d = rho_d = ux_d = uy_d = uz_d = nullptr;
    top_snd_d = bot_snd_d = top_rcv_d = bot_rcv_d = nullptr;
    topF_snd_d = botF_snd_d = topF_rcv_d = botF_rcv_d = nullptr;
    top_snd_h = bot_snd_h = top_rcv_h = bot_rcv_h = nullptr;
    topF_snd_h = botF_snd_h = topF_rcv_h = botF_rcv_h = nullptr;
    ready = false;
}

template <typename T>
T *alloc(size_t n)
{
    return static_cast<T *>(calloc(n, sizeof(T)));
}

/* cudaMemcpy on one host: a plain copy */
void copy(void *dst, const void *src, size_t bytes) { memcpy(dst, src, bytes); }

struct cwd_guard {
    char saved[4096];
    bool ok;
    explicit cwd_guard(const char *dir) { ok = getcwd(saved, sizeof(saved)) && chdir(dir) == 0; }
    ~cwd_guard()
    {
        if (ok && chdir(saved) != 0) fprintf(stderr, "zsc_ref: cannot return to %s\n", saved);
    }
};

void set_constants()
{
    /* src/main.cu:315-342 (cudaMemcpyToSymbol) */
    dcol = gridSize;
    NX = NX_h; NY = NY_h; NZ = NZ_h; NXY = NXY_h;
    K0 = Wn0; K1 = Wn1; K2 = Wn2;
    KC0 = WnC0; KC1 = WnC1; KC2 = WnC2;
    alpha4_d = alpha4; kappa_d = kappa; Gamma_d = Gamma;
    eta_d = eta; eta2_d = eta2; phiStarSq_d = phiStarSq;
    invEta2_d = invEta2; invTauPhi_d = invTauPhi; invTauPhiOne_d = invTauPhiOne;
    invTauRhoOne_d = invTauRhoOne;
    zl_d = zl; zu_d = zu;
}

}  // namespace

/* The library is built with hidden visibility (the reference defines globals
 * such as `stat`, `init` and `step` that would otherwise be bound to libc's
 * symbols of the same name when the library is loaded with dlopen); only the
 * zr_* entry points below are exported. */
#define ZR_API __attribute__((visibility("default")))

extern "C" {

/* Read dir/properties.in and dir/discrete.in, build the initial state exactly
 * as the reference driver does (src/main.cu:155-357).  phi_override, when not
 * NULL, replaces the host phi array after init() (NX*NY*(zmax+2) values
 * including both ghost planes), so that inputs with more bubbles than the
 * reference's MAX_BUBBLES can be fed in.  Returns 0 on success. */
ZR_API int zr_init(const char *dir, const float *phi_override)
{
    release();
    {
        cwd_guard g(dir);
        if (!g.ok) return 10;
        FILE *probe = fopen("properties.in", "r");
        if (!probe) return 11;
        fclose(probe);
        probe = fopen("discrete.in", "r");
        if (!probe) return 12;
        fclose(probe);
        nprocs = 1;
        proc = 0;
        RELAX = -1;
        paramRead();
        vgrid();
    }
    NX_h = xmax;
    NY_h = ymax;
    NZ_h = zug - zlg + 1;
    NXY_h = NX_h * NY_h;
    bufSize = NX_h * NY_h;
    gridSize = NX_h * NY_h * NZ_h;
    /* src/main.cu:167-173 */
    if (NX_h % 32 != 0 || NY_h % 32 != 0) return 1;
    if (BLOCK_SIZE_X * BLOCK_SIZE_Y > 512 || NX_h < BLOCK_SIZE_X || NY_h < BLOCK_SIZE_Y) return 2;
    if (nBubbles > MAX_BUBBLES) return 3;
    block_dim = zr_dim3{BLOCK_SIZE_X, BLOCK_SIZE_Y, 1};
    grid_dim = zr_dim3{NX_h / BLOCK_SIZE_X, NY_h / BLOCK_SIZE_Y, 1};

    const size_t gs = (size_t)gridSize, bs = (size_t)bufSize;
    nb_e = alloc<int>(gs); nb_w = alloc<int>(gs); nb_n = alloc<int>(gs); nb_s = alloc<int>(gs);
    phi_h = alloc<float>(gs); rho_h = alloc<float>(gs);
    ux_h = alloc<float>(gs); uy_h = alloc<float>(gs); uz_h = alloc<float>(gs);
    nb_e_d = alloc<int>(gs); nb_w_d = alloc<int>(gs); nb_n_d = alloc<int>(gs); nb_s_d = alloc<int>(gs);
    phi_d = alloc<float>(gs); rho_d = alloc<float>(gs);
    ux_d = alloc<float>(gs); uy_d = alloc<float>(gs); uz_d = alloc<float>(gs);
    for (int i = 0; i < 7; i++) f_d[i] = alloc<float>(2 * gs);
    for (int i = 0; i < 19; i++) g_d[i] = alloc<float>(2 * gs);
    top_snd_d = alloc<float>(6 * bs); bot_snd_d = alloc<float>(6 * bs);
    top_rcv_d = alloc<float>(6 * bs); bot_rcv_d = alloc<float>(6 * bs);
    topF_snd_d = alloc<float>(bs); botF_snd_d = alloc<float>(bs);
    topF_rcv_d = alloc<float>(bs); botF_rcv_d = alloc<float>(bs);
    top_snd_h = alloc<float>(6 * bs); bot_snd_h = alloc<float>(6 * bs);
    top_rcv_h = alloc<float>(6 * bs); bot_rcv_h = alloc<float>(6 * bs);
    topF_snd_h = alloc<float>(bs); botF_snd_h = alloc<float>(bs);
    topF_rcv_h = alloc<float>(bs); botF_rcv_h = alloc<float>(bs);
    if (!g_d[18] || !top_snd_h || !botF_rcv_h || !uz_d) {
        release();
        return 4;
    }

    init(nb_e, nb_w, nb_n, nb_s, phi_h, rho_h, ux_h, uy_h, uz_h);
    if (phi_override) memcpy(phi_h, phi_override, sizeof(float) * gs);

    copy(nb_e_d, nb_e, sizeof(int) * gs); copy(nb_w_d, nb_w, sizeof(int) * gs);
    copy(nb_n_d, nb_n, sizeof(int) * gs); copy(nb_s_d, nb_s, sizeof(int) * gs);
    copy(phi_d, phi_h, sizeof(float) * gs); copy(rho_d, rho_h, sizeof(float) * gs);
    copy(ux_d, ux_h, sizeof(float) * gs); copy(uy_d, uy_h, sizeof(float) * gs);
    copy(uz_d, uz_h, sizeof(float) * gs);
    set_constants();

    float **f = f_d, **g = g_d;
    launch([&] { init_f(nb_e_d, nb_w_d, nb_n_d, nb_s_d, phi_d, f[0], f[1], f[2], f[3], f[4], f[5], f[6]); });
    launch([&] {
        init_g(nb_e_d, nb_w_d, nb_n_d, nb_s_d, phi_d, rho_d, g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7],
               g[8], g[9], g[10], g[11], g[12], g[13], g[14], g[15], g[16], g[17], g[18]);
    });
    step = 0;
    ready = true;
    return 0;
}

/* nsteps iterations of the reference loop body with grav_d = grav
 * (src/main.cu:496-608; the relaxation loop is the same with grav_d = 0). */
ZR_API int zr_step(int nsteps, float grav)
{
    if (!ready) return 1;
    grav_d = grav;
    float **f = f_d, **g = g_d;
    const size_t bs = (size_t)bufSize;
    for (int t = 0; t < nsteps; t++) {
        launch([&] { update_phi(phi_d, f[0], f[1], f[2], f[3], f[4], f[5], f[6]); });
        launch([&] {
            update_rho(rho_d, g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7], g[8], g[9], g[10], g[11], g[12],
                       g[13], g[14], g[15], g[16], g[17], g[18]);
        });
        launch([&] {
            update_velocity(rho_d, ux_d, uy_d, uz_d, g[1], g[2], g[3], g[4], g[5], g[6], g[7], g[8], g[9], g[10],
                            g[11], g[12], g[13], g[14], g[15], g[16], g[17], g[18]);
        });
        launch([&] { pack_mpi_phi(topF_snd_d, botF_snd_d, phi_d); });
        copy(topF_snd_h, topF_snd_d, sizeof(float) * bs);
        copy(botF_snd_h, botF_snd_d, sizeof(float) * bs);
        mpiUpdate_phi(topF_snd_h, botF_snd_h, topF_rcv_h, botF_rcv_h);
        copy(topF_rcv_d, topF_rcv_h, sizeof(float) * bs);
        copy(botF_rcv_d, botF_rcv_h, sizeof(float) * bs);
        launch([&] { unpack_mpi_phi(topF_rcv_d, botF_rcv_d, phi_d); });

        launch([&] {
            collision_f(nb_e_d, nb_w_d, nb_n_d, nb_s_d, phi_d, rho_d, ux_d, uy_d, uz_d, f[0], f[1], f[2], f[3],
                        f[4], f[5], f[6]);
        });
        launch([&] {
            collision_g(nb_e_d, nb_w_d, nb_n_d, nb_s_d, phi_d, rho_d, ux_d, uy_d, uz_d, g[0], g[1], g[2], g[3],
                        g[4], g[5], g[6], g[7], g[8], g[9], g[10], g[11], g[12], g[13], g[14], g[15], g[16],
                        g[17], g[18]);
        });

        launch([&] { pack_mpi_f(topF_snd_d, botF_snd_d, f[5], f[6]); });
        copy(topF_snd_h, topF_snd_d, sizeof(float) * bs);
        copy(botF_snd_h, botF_snd_d, sizeof(float) * bs);
        mpiUpdate_f(topF_snd_h, botF_snd_h, topF_rcv_h, botF_rcv_h);
        copy(topF_rcv_d, topF_rcv_h, sizeof(float) * bs);
        copy(botF_rcv_d, botF_rcv_h, sizeof(float) * bs);
        launch([&] { unpack_mpi_f(topF_rcv_d, botF_rcv_d, f[5], f[6]); });

        launch([&] { stream_f(nb_e_d, nb_w_d, nb_n_d, nb_s_d, f[0], f[1], f[2], f[3], f[4], f[5], f[6]); });
        launch([&] {
            stream_g(nb_e_d, nb_w_d, nb_n_d, nb_s_d, g[0], g[1], g[2], g[3], g[4], g[5], g[6], g[7], g[8], g[9],
                     g[10], g[11], g[12], g[13], g[14], g[15], g[16], g[17], g[18]);
        });

        launch([&] {
            pack_mpi(top_snd_d, bot_snd_d, f[5], f[6], g[5], g[6], g[11], g[12], g[13], g[14], g[15], g[16],
                     g[17], g[18]);
        });
        copy(top_snd_h, top_snd_d, sizeof(float) * 6 * bs);
        copy(bot_snd_h, bot_snd_d, sizeof(float) * 6 * bs);
        mpiUpdate(top_snd_h, bot_snd_h, top_rcv_h, bot_rcv_h);
        copy(top_rcv_d, top_rcv_h, sizeof(float) * 6 * bs);
        copy(bot_rcv_d, bot_rcv_h, sizeof(float) * 6 * bs);
        launch([&] {
            unpack_mpi(top_rcv_d, bot_rcv_d, f[5], f[6], g[5], g[6], g[11], g[12], g[13], g[14], g[15], g[16],
                       g[17], g[18]);
        });
        step++;
    }
    return 0;
}

/* Interior planes (k = 1 .. NZ-2) of the reference's phi, rho, u arrays;
 * each output holds NX*NY*zmax values, x fastest.  NULL pointers are skipped. */
ZR_API int zr_fields(float *phi, float *rho, float *ux, float *uy, float *uz)
{
    if (!ready) return 1;
    const size_t plane = (size_t)NXY_h, nin = plane * (size_t)(NZ_h - 2);
    float *src[5] = {phi_d, rho_d, ux_d, uy_d, uz_d};
    float *dst[5] = {phi, rho, ux, uy, uz};
    for (int i = 0; i < 5; i++)
        if (dst[i]) memcpy(dst[i], src[i] + plane, sizeof(float) * nin);
    return 0;
}

/* Interior planes of the current (lower-half) distributions: f as 7 blocks,
 * g as 19 blocks of NX*NY*zmax values. */
ZR_API int zr_dist(float *f, float *g)
{
    if (!ready) return 1;
    const size_t plane = (size_t)NXY_h, nin = plane * (size_t)(NZ_h - 2);
    for (int i = 0; i < 7; i++)
        if (f) memcpy(f + i * nin, f_d[i] + plane, sizeof(float) * nin);
    for (int i = 0; i < 19; i++)
        if (g) memcpy(g + i * nin, g_d[i] + plane, sizeof(float) * nin);
    return 0;
}

/* {xmax, ymax, zmax, NZ (with ghosts), nBubbles, maxStep, relaxStep, save, stat, BLOCK_SIZE_X, BLOCK_SIZE_Y} */
ZR_API int zr_dims(int *out)
{
    int v[11] = {xmax, ymax, zmax, NZ_h, nBubbles, maxStep, relaxStep, save, stat, BLOCK_SIZE_X, BLOCK_SIZE_Y};
    memcpy(out, v, sizeof(v));
    return 0;
}

/* Derived constants of src/paramread.c:141-170 as the reference computed them (float):
 * {phiStar, phiStarSq, invTauRhoOne, eta, eta2, invEta2, invTauPhi, invTauPhiOne,
 *  alpha, alpha4, kappa, gravity, grav, Wn0, Wn1, Wn2, WnC0, WnC1, WnC2} */
ZR_API int zr_consts(float *out)
{
    float v[19] = {phiStar, phiStarSq, invTauRhoOne, eta, eta2, invEta2, invTauPhi, invTauPhiOne,
                   alpha, alpha4, kappa, gravity, grav, Wn0, Wn1, Wn2, WnC0, WnC1, WnC2};
    memcpy(out, v, sizeof(v));
    return 0;
}

/* Run the reference's own stats() (src/stats.c) and, if with_log, the
 * relaxation block of logSave() (src/logsave.c:241-252) in dir, on the current
 * fields.  relax: 1 = relaxation stage (relax_stats.out), 0 = evolution stage
 * (stats.out).  step_no = 0 starts a new stats file. */
ZR_API int zr_write_stats(const char *dir, int relax, int step_no, int with_log)
{
    if (!ready) return 1;
    cwd_guard g(dir);
    if (!g.ok) return 10;
    const size_t gs = (size_t)gridSize;
    copy(phi_h, phi_d, sizeof(float) * gs);
    copy(rho_h, rho_d, sizeof(float) * gs);
    copy(ux_h, ux_d, sizeof(float) * gs);
    copy(uy_h, uy_d, sizeof(float) * gs);
    copy(uz_h, uz_d, sizeof(float) * gs);
    const int saved_step = step;
    RELAX = relax;
    step = step_no;
    stats(phi_h, ux_h, uy_h, uz_h);
    if (with_log && relax == 1) {
        char name[] = "cpu-emulated";
        logSave(name, 0.f, nb_e, nb_w, nb_n, nb_s, phi_h, rho_h, ux_h, uy_h, uz_h);
    }
    step = saved_step;
    return 0;
}

ZR_API int zr_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

ZR_API void zr_free(void) { release(); }

}  /* extern "C" */
