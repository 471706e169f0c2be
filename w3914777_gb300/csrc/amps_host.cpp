// amps_host.cpp -- host-only parts of the C ABI: parameter presets, parameter
// validation and initial states.  Needs no GPU.
#include "../../include/amps.h"

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <vector>

namespace {

uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// Counter-based uniform in [0,1): the splitmix64 finaliser (Steele, Lea &
// Flood 2014) of (seed, a, b).  The same function drives the device noise.
double u01(uint64_t seed, uint64_t a, uint64_t b)
{
    return (double)(mix64(mix64(seed ^ mix64(a)) + b) >> 11) * 0x1.0p-53;
}

void base(amps_params *p, int model)
{
    memset(p, 0, sizeof(*p));
    p->model = model;
    p->mode = AMPS_PUREHIGH;
    p->nx = p->ny = 512;           // snowflake/paras/total.h:20
    p->tile = 16;                  // snowflake/paras/total.h:21
    p->bc = AMPS_BC_PERIODIC;
    p->high_tier = AMPS_TIER_FP64; // sweep scripts' "typedef double highprecision"
    p->monitor = AMPS_MONITOR_TEM; // snowflake/paras/total.h:28 (#define Monitor2)
    p->monitor_samples = 0;
    p->monitor_field = model == AMPS_GRAINGROWTH ? 1 : 0;  // eta2 (graingrowth/end2end_mix.cu:83); phi; c
    p->cadence = 10;               // snowflake/end2end_mix.cu:87
    p->thr_lo = p->thr_hi = 0.99;  // snowflake/paras/total.h:22
    p->gram_ratio = 1.0;           // snowflake/paras/total.h:23
    p->ref_order = 1;
    p->mu_lap_fp64 = 1;
    p->pi = 3.1415926;             // snowflake/paras/total.h:47
    p->seed = 1234;
}

}  // namespace

extern "C" int amps_abi_version(void) { return AMPS_ABI_VERSION; }

extern "C" int amps_num_fields(const amps_params *p)
{
    if (!p) return -1;
    if (p->model == AMPS_KOBAYASHI) return 2;
    if (p->model == AMPS_GRAINGROWTH) return p->nfields;
    if (p->model == AMPS_SINTERING) return p->nfields + 1;
    return -1;
}

extern "C" int amps_preset(int model, int preset, amps_params *p)
{
    if (!p || model < 0 || model > 2 || preset < 0 || preset > 5) return AMPS_ERR_INVALID;
    base(p, model);
    if (model == AMPS_KOBAYASHI) {
        // snowflake/paras/para1-5.h
        static const double aniso[5] = {4.0, 6.0, 5.0, 6.0, 4.0};
        static const double theta0[5] = {0.0, 0.0, 0.0, 0.4, 0.25};
        p->nfields = 2;
        p->dx = p->dy = 0.03;
        p->tau = 0.0003; p->epsb = 0.01; p->kappa = 1.8; p->delta = 0.02;
        p->alpha = 0.9; p->gama = 10.0; p->teq = 1.0; p->dt = 1.0e-4;
        p->init_r2 = 10.0;   // `seed` in para*.h, compared with r^2 (snowflake/tools.h:29)
        p->init_offset = 8;  // disc centre (dimX/2+8, dimY/2+8), snowflake/tools.h:28
        if (preset >= 1) {
            p->aniso = aniso[preset - 1];
            p->theta0 = theta0[preset - 1];
        } else {
            // seeded 512^2 dendrite: zero flux, theta0=0.2, K=1.6, disc r=5 at the centre, noise 0.01
            p->aniso = 6.0; p->theta0 = 0.2; p->kappa = 1.6;
            p->bc = AMPS_BC_NOFLUX;
            p->init_r2 = 25.0; p->init_offset = 0;
            p->noise = 0.01;
            p->tile = 32;
        }
    } else if (model == AMPS_GRAINGROWTH) {
        // graingrowth/paras/para1-5.h
        static const double mobil[5] = {5.0, 10.0, 5.0, 5.0, 20.0};
        static const double grcoef[5] = {0.1, 0.1, 0.2, 0.1, 0.1};
        static const double R[5] = {50, 50, 50, 80, 50};
        p->nfields = 2;
        p->gamma = 1.0;  // the reference's 2.0*1.0 (graingrowth/function.h:22)
        p->dx = p->dy = 0.5; p->dt = 0.005;
        if (preset >= 1) {
            p->mobil = mobil[preset - 1];
            p->grcoef = grcoef[preset - 1];
            p->init_r = R[preset - 1];
        } else {
            // Fan-Chen 1024^2, Q=8, gamma=1.5, kappa=2, L=1, dx=1, dt=0.05, eta ~ U[-1e-3,1e-3]
            p->nx = p->ny = 1024;
            p->nfields = 8;
            p->gamma = 1.5; p->grcoef = 2.0; p->mobil = 1.0;
            p->dx = p->dy = 1.0; p->dt = 0.05;
            p->init_amp = 1e-3;
            p->tile = 32;
            p->mode = AMPS_END2END_MIX;
            p->monitor = AMPS_MONITOR_SPA;
            p->monitor_samples = 1;
            p->monitor_field = -1;
            p->thr_lo = 0.02;
            p->thr_hi = 1.2;
            p->ref_order = 0;
        }
    } else {
        // sintering/paras/para1-5.h
        static const double coefm[5] = {5.0, 5.0, 20.0, 20.0, 20.0};
        static const double dsur[5] = {32, 64, 16, 16, 64};
        static const double R1[5] = {50, 50, 50, 20, 20};
        p->nfields = 2;
        p->coefk = 2.0; p->coefl = 5.0; p->dvol = 0.040; p->dvap = 0.002; p->dgrb = 1.6;
        p->dx = p->dy = 0.5; p->dt = 1.0e-4;
        p->A = 16.0; p->B = 1.0;  // sintering/function.h:70 (2.0*16.0, 1.0*)
        if (preset >= 1) {
            p->coefm = coefm[preset - 1];
            p->dsur = dsur[preset - 1];
            p->init_r = R1[preset - 1];
        } else {
            // 1024^2, 16 particles r in [20,40]: A=16 B=1 kc=5 ke=2 Dvol=.04 Dvap=.002 Ds=16 Dgb=1.6 L=10
            p->nx = p->ny = 1024;
            p->nfields = 16;
            p->coefm = 5.0; p->coefk = 2.0; p->coefl = 10.0; p->dsur = 16.0;
            p->rmin = 20; p->rmax = 40;
            p->tile = 32;
            p->mode = AMPS_END2END_MIX;
            p->monitor = AMPS_MONITOR_SPA;
            p->monitor_samples = 1;
            p->thr_lo = 0.02;
            p->thr_hi = 0.5;
            p->ref_order = 0;
        }
    }
    return AMPS_OK;
}

extern "C" int amps_check_params(const amps_params *p, char *msg, size_t len)
{
    char buf[256] = {0};
#define BAD(...)                                  \
    do {                                          \
        snprintf(buf, sizeof buf, __VA_ARGS__);   \
        if (msg && len) snprintf(msg, len, "%s", buf); \
        return AMPS_ERR_INVALID;                  \
    } while (0)
    if (!p) BAD("params is NULL");
    if (p->model < 0 || p->model > 2) BAD("unknown model %d", p->model);
    if (p->mode < 0 || p->mode > 4) BAD("unknown mode %d", p->mode);
    if (p->tile != 16 && p->tile != 32) BAD("tile must be 16 or 32 (got %d)", p->tile);
    if (p->nx < p->tile || p->ny < p->tile)
        BAD("nx, ny (%d, %d) must be at least the tile (%d)", p->nx, p->ny, p->tile);
    // ragged grids (a side not a multiple of the tile): grain growth only;
    // storage keeps whole tiles and the edge tiles compute their valid cells
    const bool ragged = p->nx % p->tile || p->ny % p->tile;
    if (ragged && p->model != AMPS_GRAINGROWTH)
        BAD("nx, ny (%d, %d) must be multiples of the tile (%d) for Kobayashi and sintering "
            "(grain growth takes any sides)", p->nx, p->ny, p->tile);
    if (ragged && p->half_arith != AMPS_HALF_FP32)
        BAD("binary16 half-tile arithmetic needs sides that are multiples of the tile");
    if (ragged && p->ref_snapshot) BAD("the reference's snapshot rule needs sides that are multiples of the tile");
    const int64_t ntx = (p->nx + p->tile - 1) / p->tile, nty = (p->ny + p->tile - 1) / p->tile;
    if (ntx * nty * p->tile * p->tile > (int64_t)1 << 31) BAD("grid too large");
    // the classification ranks each tier's tiles in a 21-bit field of one
    // packed 64-bit counter (three tiers per scan)
    if (ntx * nty > AMPS_MAX_TILES)
        BAD("too many tiles (%lld > %lld): use the larger tile", (long long)(ntx * nty), (long long)AMPS_MAX_TILES);
    if (p->bc != AMPS_BC_PERIODIC && p->bc != AMPS_BC_NOFLUX) BAD("unknown boundary condition %d", p->bc);
    if (p->high_tier != AMPS_TIER_FP64 && p->high_tier != AMPS_TIER_FP32) BAD("high_tier must be FP64 or FP32");
    if (p->model == AMPS_GRAINGROWTH && (p->nfields < 1 || p->nfields > 32)) BAD("grain growth Q must be 1..32");
    if (p->model == AMPS_SINTERING && (p->nfields < 1 || p->nfields > 32)) BAD("sintering N must be 1..32");
    if (p->monitor < AMPS_MONITOR_SPA || p->monitor > AMPS_MONITOR_RATE) BAD("monitor must be 1, 2 or 3");
    const int nf = amps_num_fields(p);
    if (p->monitor_field < -1 || p->monitor_field >= nf) BAD("monitor_field out of range");
    if (p->cadence < 1) BAD("cadence must be >= 1");
    if (!(p->thr_lo <= p->thr_hi)) BAD("thr_lo must be <= thr_hi");
    if (!(p->dx > 0) || !(p->dy > 0) || !(p->dt > 0)) BAD("dx, dy, dt must be positive");
    if (p->mode == AMPS_GRAM1 || p->mode == AMPS_GRAM2)
        if (!(p->gram_ratio >= 0 && p->gram_ratio <= 1)) BAD("gram_ratio must be in [0,1]");
    if (p->half_arith < AMPS_HALF_FP32 || p->half_arith > AMPS_HALF_SR) BAD("half_arith must be 0, 1, 2 or 3");
    if (p->half_arith == AMPS_HALF_SR && p->model != AMPS_KOBAYASHI)
        BAD("stochastic rounding of half tiles is built for Kobayashi only");
    if (p->half_arith == AMPS_HALF_HFMA2 && p->model != AMPS_GRAINGROWTH)
        BAD("the HFMA2 half arithmetic is built for grain growth only");
    if (p->half_arith == AMPS_HALF_REF && p->model == AMPS_KOBAYASHI)
        BAD("the reference's half arithmetic is built for grain growth and sintering (Kobayashi's needs "
            "device-only half transcendentals)");
    if (p->half_arith == AMPS_HALF_REF && p->model == AMPS_SINTERING &&
        (p->high_tier != AMPS_TIER_FP64 || (p->mode == AMPS_END2END_MIX && p->thr_lo != p->thr_hi)))
        BAD("sintering with the reference's half arithmetic has the reference's two tiers: half and FP64 "
            "(high_tier FP64, thr_lo == thr_hi)");
    if (p->ref_snapshot != 0 && p->ref_snapshot != 1) BAD("ref_snapshot must be 0 or 1");
    if (msg && len) msg[0] = 0;
    return AMPS_OK;
#undef BAD
}

namespace {

// Seeded touching-cluster placement of N discs (radii integer in [rmin, rmax]):
// each new disc touches a random earlier one and overlaps none.
bool place_particles(const amps_params *p, std::vector<double> &cx, std::vector<double> &cy,
                     std::vector<double> &r)
{
    const int np = p->nfields;
    uint64_t k = 0;
    auto U = [&]() { return u01(p->seed, 0x53494E54ull, k++); };
    const int span = (int)(p->rmax - p->rmin) + 1;
    for (int i = 0; i < np; ++i) r.push_back(p->rmin + (span > 0 ? floor(U() * span) : 0));
    cx.push_back(p->nx / 2.0);
    cy.push_back(p->ny / 2.0);
    for (int i = 1; i < np; ++i) {
        bool ok = false;
        for (int att = 0; att < 100000 && !ok; ++att) {
            const int j = (int)floor(U() * i);
            const double th = 2.0 * M_PI * U();
            const double x = cx[j] + (r[i] + r[j]) * cos(th), y = cy[j] + (r[i] + r[j]) * sin(th);
            if (x - r[i] < 2 || y - r[i] < 2 || x + r[i] > p->nx - 2 || y + r[i] > p->ny - 2) continue;
            ok = true;
            for (int m = 0; m < i && ok; ++m)
                if (m != j && hypot(x - cx[m], y - cy[m]) < r[i] + r[m]) ok = false;
            if (ok) { cx.push_back(x); cy.push_back(y); }
        }
        if (!ok) return false;
    }
    return true;
}

}  // namespace

extern "C" int amps_init_host(const amps_params *p, int kind, double *const *fields)
{
    if (amps_check_params(p, nullptr, 0) != AMPS_OK || !fields) return AMPS_ERR_INVALID;
    if (kind != AMPS_INIT_REFERENCE && kind != AMPS_INIT_SEEDED) return AMPS_ERR_INVALID;
    const int nx = p->nx, ny = p->ny, nf = amps_num_fields(p);
    const int64_t n = (int64_t)nx * ny;
    for (int f = 0; f < nf; ++f) memset(fields[f], 0, n * sizeof(double));
    if (p->model == AMPS_KOBAYASHI) {
        // snowflake/tools.h:24-33 (float distance, phi=1 where r^2 < seed)
        const int cx = nx / 2 + p->init_offset, cy = ny / 2 + p->init_offset;
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                float d = (float)(pow((double)(x - cx), 2) + pow((double)(y - cy), 2));
                fields[0][(int64_t)y * nx + x] = d < (float)p->init_r2 ? 1.0 : 0.0;
            }
    } else if (p->model == AMPS_GRAINGROWTH) {
        if (kind == AMPS_INIT_REFERENCE) {
            // graingrowth/tools.h:24-38: eta2=1 inside R about the centre, eta1=1 outside
            const float rx = (float)(nx / 2), ry = (float)(ny / 2), R = (float)p->init_r;
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x) {
                    float d = (float)sqrt(pow(x - rx, 2) + pow(y - ry, 2));
                    const int64_t i = (int64_t)y * nx + x;
                    if (nf >= 2) {
                        fields[0][i] = d <= R ? 0.0 : 1.0;
                        fields[1][i] = d <= R ? 1.0 : 0.0;
                    } else {
                        fields[0][i] = d <= R ? 1.0 : 0.0;
                    }
                }
        } else {
            for (int f = 0; f < nf; ++f)
                for (int64_t i = 0; i < n; ++i) fields[f][i] = p->init_amp * (2.0 * u01(p->seed, (uint64_t)f, (uint64_t)i) - 1.0);
        }
    } else {
        if (kind == AMPS_INIT_REFERENCE) {
            // sintering/main.cu:45-59 and sintering/paras/para*.h:6-7 (R2 = R1/2,
            // Ry1 = 240 for 512 rows, Ry2 = Ry1+R1+R2, Rx1 = dimX/2+8), 1-based indices
            const float R1 = (float)p->init_r, R2 = R1 / 2;
            const float Ry1 = (float)(ny / 2 - 16), Ry2 = Ry1 + R1 + R2, Rx1 = (float)(nx / 2 + 8);
            for (int y = 1; y <= ny; ++y)
                for (int x = 1; x <= nx; ++x) {
                    float d1 = (float)sqrt(pow(x - Rx1, 2) + pow(y - Ry1, 2));
                    float d2 = (float)sqrt(pow(x - Rx1, 2) + pow(y - Ry2, 2));
                    const int64_t i = (int64_t)(y - 1) * nx + x - 1;
                    if (d1 <= R1) { fields[0][i] = 1; if (nf > 1) fields[1][i] = 1; }
                    if (d2 <= R2) { fields[0][i] = 1; if (nf > 2) fields[2][i] = 1; if (nf > 1) fields[1][i] = 0.0; }
                }
        } else {
            std::vector<double> cx, cy, r;
            if (!place_particles(p, cx, cy, r)) return AMPS_ERR_INVALID;
            for (int y = 1; y <= ny; ++y)
                for (int x = 1; x <= nx; ++x) {
                    const int64_t i = (int64_t)(y - 1) * nx + x - 1;
                    for (int k = 0; k < (int)r.size(); ++k)
                        if (hypot(x - cx[k], y - cy[k]) <= r[k]) {
                            fields[0][i] = 1;
                            for (int m = 1; m < nf; ++m) fields[m][i] = 0.0;
                            fields[k + 1][i] = 1;
                        }
                }
        }
    }
    return AMPS_OK;
}
