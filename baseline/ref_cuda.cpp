// ref_cuda.cpp -- host driver of the reference's own CUDA kernels on the GPU.
//
// The reference's device code is built in place from its read-only tree into
// cubins (baseline/Makefile, `make cubins`: graingrowth/function.h and
// tools.h with the header settings its sweep scripts write).  Its host
// programs are not built: they fix sizes at compile time and write results
// to files.  This file restates their time loops -- the same kernels, launch
// shapes, argument lists, device synchronisations and event timing -- around
// driver-API launches of the reference's kernels, found in the cubin by name:
//   refcuda_gg_pure:  graingrowth/purehigh.cu:14-45 (End2end)
//   refcuda_gg_mix:   graingrowth/end2end_mix.cu:31-105 (AMSTENCIL)
//   refcuda_kob_pure: snowflake/purehigh.cu:13-36 (End2end)
//   refcuda_kob_mix:  snowflake/end2end_mix.cu:30-112 (AMSTENCIL)
//   refcuda_gg_purelow:  graingrowth/purelow.cu:3-47 (HALF2)
//   refcuda_kob_purelow: snowflake/purelow.cu:3-66 (HALF2)
//   refcuda_sint_pure, refcuda_sint_mix: sintering/main.cu:44-206 (PURE,
//     AMSTENCIL); the initial state (main.cu:45-59, a host loop) comes from
//     the caller, and the classification at a run-time threshold from the
//     wrapper's restated get_type (ref_get_type_rt)
// The reference allocates with cudaMallocManaged, whose pages the first
// touch zero-fills; here device allocations are zeroed explicitly.  The
// elapsed time is the reference's own: CUDA events from step 5 to the end.
#include <cuda.h>
#include <cuda_fp16.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

namespace {

std::string g_err;

struct RefModule {
    CUcontext ctx = nullptr;
    CUmodule mod = nullptr;
    int dims[4] = {0, 0, 0, 0};  // dimX, dimY, unitx, unity
    std::map<std::string, CUfunction> fns;
};

bool ck(CUresult r, const char *what)
{
    if (r == CUDA_SUCCESS) return true;
    const char *s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "unknown error");
    return false;
}

// The kernel named `name` (a C++ function at namespace scope: its mangled
// name starts with _Z<length><name> and the parameter types follow).
CUfunction kernel(RefModule *m, const char *name)
{
    auto it = m->fns.find(name);
    if (it != m->fns.end()) return it->second;
    unsigned count = 0;
    if (!ck(cuModuleGetFunctionCount(&count, m->mod), "cuModuleGetFunctionCount")) return nullptr;
    std::vector<CUfunction> all(count);
    if (!ck(cuModuleEnumerateFunctions(all.data(), count, m->mod), "cuModuleEnumerateFunctions")) return nullptr;
    // the length prefix fixes the name: any function whose mangled name
    // starts with _Z<length><name> is `name` (the parameter codes follow)
    const std::string prefix = "_Z" + std::to_string(strlen(name)) + name;
    for (CUfunction f : all) {
        const char *fn = nullptr;
        if (cuFuncGetName(&fn, f) != CUDA_SUCCESS || !fn) continue;
        // (or an extern "C" kernel of the wrapper, by its plain name)
        if (strncmp(fn, prefix.c_str(), prefix.size()) == 0 || strcmp(fn, name) == 0) {
            m->fns[name] = f;
            return f;
        }
    }
    g_err = std::string("kernel not in the cubin: ") + name;
    return nullptr;
}

struct Dim {
    unsigned x, y, z;
};

bool launch(RefModule *m, const char *name, Dim g, Dim b, std::vector<void *> args)
{
    CUfunction f = kernel(m, name);
    if (!f) return false;
    return ck(cuLaunchKernel(f, g.x, g.y, g.z, b.x, b.y, b.z, 0, nullptr, args.data(), nullptr), name);
}

// Zeroed device buffers, freed together.
struct Buffers {
    std::vector<CUdeviceptr> all;
    ~Buffers()
    {
        for (CUdeviceptr p : all) cuMemFree(p);
    }
    bool get(CUdeviceptr &p, size_t bytes)
    {
        if (!ck(cuMemAlloc(&p, bytes), "cuMemAlloc")) return false;
        all.push_back(p);
        return ck(cuMemsetD8(p, 0, bytes), "cuMemsetD8");
    }
};

// Elapsed ms between two events recorded on the default stream.
struct Timer {
    CUevent a = nullptr, b = nullptr;
    bool started = false;
    ~Timer()
    {
        if (a) cuEventDestroy(a);
        if (b) cuEventDestroy(b);
    }
    bool start()
    {
        if (!ck(cuEventCreate(&a, CU_EVENT_DEFAULT), "cuEventCreate") ||
            !ck(cuEventCreate(&b, CU_EVENT_DEFAULT), "cuEventCreate"))
            return false;
        started = true;
        return ck(cuEventRecord(a, nullptr), "cuEventRecord");
    }
    bool stop(float *ms)
    {
        *ms = 0.f;
        if (!started) return true;
        return ck(cuEventRecord(b, nullptr), "cuEventRecord") && ck(cuEventSynchronize(b), "cuEventSynchronize") &&
               ck(cuEventElapsedTime(ms, a, b), "cuEventElapsedTime");
    }
};

bool current(RefModule *m) { return ck(cuCtxSetCurrent(m->ctx), "cuCtxSetCurrent"); }

}  // namespace

extern "C" {

const char *refcuda_error(void) { return g_err.c_str(); }

// Load a cubin into the device's primary context (the one the CUDA runtime
// uses too); nullptr on failure (refcuda_error).
void *refcuda_open(const char *cubin)
{
    CUdevice dev;
    auto *m = new RefModule();
    if (!ck(cuInit(0), "cuInit") || !ck(cuDeviceGet(&dev, 0), "cuDeviceGet") ||
        !ck(cuDevicePrimaryCtxRetain(&m->ctx, dev), "cuDevicePrimaryCtxRetain") || !current(m) ||
        !ck(cuModuleLoad(&m->mod, cubin), "cuModuleLoad")) {
        delete m;
        return nullptr;
    }
    CUdeviceptr p;
    size_t bytes = 0;
    if (!ck(cuModuleGetGlobal(&p, &bytes, m->mod, "ref_dims"), "ref_dims") || bytes != sizeof m->dims ||
        !ck(cuMemcpyDtoH(m->dims, p, sizeof m->dims), "ref_dims")) {
        cuModuleUnload(m->mod);
        delete m;
        return nullptr;
    }
    return m;
}

void refcuda_close(void *h)
{
    auto *m = static_cast<RefModule *>(h);
    if (!m) return;
    current(m);
    cuModuleUnload(m->mod);
    CUdevice dev;
    if (cuCtxGetDevice(&dev) == CUDA_SUCCESS) cuDevicePrimaryCtxRelease(dev);
    delete m;
}

// The build's compile-time sizes: dimX, dimY, unitx, unity.
void refcuda_dims(void *h, int *out)
{
    memcpy(out, static_cast<RefModule *>(h)->dims, sizeof(int) * 4);
}

// graingrowth/purehigh.cu:14-45 for `steps` steps: dataprepare_high, then
// per step kernel1_pure for eta1 and for eta2 (each from the old pair), a
// device synchronisation and the swap.  eta1, eta2 (host, dimX*dimY): the
// fields at the end; ms: the reference's elapsed time from step 5.
int refcuda_gg_pure(void *h, int steps, double *eta1_host, double *eta2_host, float *ms)
{
    auto *m = static_cast<RefModule *>(h);
    if (!m || !current(m)) return 1;
    const int nx = m->dims[0], ny = m->dims[1], ux = m->dims[2], uy = m->dims[3];
    const size_t bytes = sizeof(double) * nx * ny;
    const unsigned tiles = (unsigned)((nx / ux) * (ny / uy));
    Buffers B;
    CUdeviceptr eta1, eta2, eta1_out, eta2_out, eta1_lap, eta2_lap, dfdeta1, dfdeta2;
    for (CUdeviceptr *p : {&eta1, &eta2, &eta1_out, &eta2_out, &eta1_lap, &eta2_lap, &dfdeta1, &dfdeta2})
        if (!B.get(*p, bytes)) return 1;
    const Dim blocks{(unsigned)ux, (unsigned)uy, 1}, grids{1, 1, tiles};
    if (!launch(m, "dataprepare_high", grids, blocks, {&eta1, &eta2}) || !ck(cuCtxSynchronize(), "sync")) return 1;
    Timer t;
    for (int i = 0; i < steps; ++i) {
        if (i == 5 && !t.start()) return 1;
        if (!launch(m, "kernel1_pure", grids, blocks, {&eta1, &eta2, &eta1_lap, &dfdeta1, &eta1_out}) ||
            !launch(m, "kernel1_pure", grids, blocks, {&eta2, &eta1, &eta2_lap, &dfdeta2, &eta2_out}) ||
            !ck(cuCtxSynchronize(), "sync"))
            return 1;
        std::swap(eta1, eta1_out);
        std::swap(eta2, eta2_out);
    }
    if (!t.stop(ms)) return 1;
    if (eta1_host && !ck(cuMemcpyDtoH(eta1_host, eta1, bytes), "copy")) return 1;
    if (eta2_host && !ck(cuMemcpyDtoH(eta2_host, eta2, bytes), "copy")) return 1;
    return 0;
}

// graingrowth/end2end_mix.cu:31-105 (AMSTENCIL) for `steps` steps at
// threshold `thr` with the cubin's monitor (`monitor`: 1 get_max_diff1, 2
// get_max_diff2 -- the build's Monitor1/Monitor2).  types (host, may be
// null): [ceil(steps/10)][tiles] uint8, type_curr after each classification
// (1 = half2, 2 = high); eta1, eta2 (host): the high arrays at the end with
// the half tiles gathered (data_sychro_aftercomputation); ms: the
// reference's elapsed time from step 5.
int refcuda_gg_mix(void *h, int steps, double thr, int monitor, double *eta1_host, double *eta2_host,
                   unsigned char *types, float *ms)
{
    auto *m = static_cast<RefModule *>(h);
    if (!m || !current(m) || (monitor != 1 && monitor != 2)) return 1;
    const int nx = m->dims[0], ny = m->dims[1], ux = m->dims[2], uy = m->dims[3];
    const int ntx = nx / ux, nty = ny / uy, tiles = ntx * nty, uxd2 = ux / 2;
    const size_t n = (size_t)nx * ny, bytes = sizeof(double) * n, hbytes = sizeof(__half) * n;
    {
        CUdeviceptr p;
        size_t sz = 0;
        if (!ck(cuModuleGetGlobal(&p, &sz, m->mod, "threshold"), "threshold") || sz != sizeof(double) ||
            !ck(cuMemcpyHtoD(p, &thr, sizeof thr), "threshold"))
            return 1;
    }
    Buffers B;
    CUdeviceptr eta1, eta2, eta1_lap, eta2_lap, dfdeta1, dfdeta2, eta1_out, eta2_out, eta2_last;
    for (CUdeviceptr *p : {&eta1, &eta2, &eta1_out, &eta2_out, &eta1_lap, &eta2_lap, &dfdeta1, &dfdeta2, &eta2_last})
        if (!B.get(*p, bytes)) return 1;
    CUdeviceptr heta1, heta2, heta1_lap, heta2_lap, hdfdeta1, hdfdeta2, heta1_out, heta2_out, type_curr, type_old,
        max_diff;
    for (CUdeviceptr *p : {&heta1, &heta2, &heta1_out, &heta2_out, &heta1_lap, &heta2_lap, &hdfdeta1, &hdfdeta2})
        if (!B.get(*p, hbytes)) return 1;
    if (!B.get(type_curr, sizeof(int) * tiles) || !B.get(type_old, sizeof(int) * tiles) ||
        !B.get(max_diff, sizeof(double) * tiles))
        return 1;
    const Dim tile_grid{1, 1, (unsigned)tiles};
    if (!launch(m, "dataprepare_high", tile_grid, Dim{(unsigned)ux, (unsigned)uy, 1}, {&eta1, &eta2}) ||
        !ck(cuCtxSynchronize(), "sync") ||
        !launch(m, "dataprepare_half2", tile_grid, Dim{(unsigned)uxd2, (unsigned)uy, 1}, {&heta1, &heta2}) ||
        !ck(cuCtxSynchronize(), "sync"))
        return 1;
    if (monitor == 2) {  // eta2_last = (eta2 == 0), end2end_mix.cu:43-47
        std::vector<double> v(n);
        if (!ck(cuMemcpyDtoH(v.data(), eta2, bytes), "copy")) return 1;
        for (double &x : v) x = x == 0 ? 1.0 : 0.0;
        if (!ck(cuMemcpyHtoD(eta2_last, v.data(), bytes), "copy")) return 1;
    }
    const Dim blocks_detect{(unsigned)(ntx > 32 ? 32 : ntx), (unsigned)(nty > 32 ? 32 : nty), 1};
    const Dim grids_detect{(unsigned)(ntx > 32 ? ntx / 32 : 1), (unsigned)(nty > 32 ? nty / 32 : 1), 1};
    const Dim sync_blocks{(unsigned)uxd2, (unsigned)uy, 1};
    // the half2 constants, end2end_mix.cu:57-66 (TOLOW = __float2half2_rn of
    // the build's double constants: mobil, grcoef, dx, dy, dxdy, dtime)
    double c[6];
    {
        CUdeviceptr p;
        size_t sz = 0;
        if (!ck(cuModuleGetGlobal(&p, &sz, m->mod, "ref_consts"), "ref_consts") || sz != sizeof c ||
            !ck(cuMemcpyDtoH(c, p, sizeof c), "ref_consts"))
            return 1;
    }
    __half2 hmobil = __float2half2_rn(c[0]), hgrcoef = __float2half2_rn(c[1]), hdxdy = __float2half2_rn(c[4]),
            height = __float2half2_rn(8.0), hdtime = __float2half2_rn(c[5]), hone = __float2half2_rn(1.0),
            htwo = __float2half2_rn(2.0);
    const Dim blocks_mix{(unsigned)uxd2, (unsigned)uy, 1}, grids_mix{2, 1, (unsigned)tiles};
    Timer t;
    int period = 0;
    std::vector<int> tc(tiles);
    for (int i = 0; i < steps; ++i) {
        if (i == 5 && !t.start()) return 1;
        if (i % 10 == 0) {
            const bool ok = monitor == 1 ? launch(m, "get_max_diff1", grids_detect, blocks_detect, {&eta2, &max_diff})
                                         : launch(m, "get_max_diff2", grids_detect, blocks_detect,
                                                  {&eta2_last, &eta2, &max_diff});
            if (!ok || !launch(m, "get_type", grids_detect, blocks_detect, {&max_diff, &type_old, &type_curr}) ||
                !ck(cuCtxSynchronize(), "sync") ||
                !launch(m, "data_sychro_duringcomputation", tile_grid, sync_blocks,
                        {&eta1, &eta2, &heta1, &heta2, &type_old, &type_curr}) ||
                !ck(cuCtxSynchronize(), "sync"))
                return 1;
            if (types) {
                // outside the reference's loop: read the classification for the caller
                if (!ck(cuMemcpyDtoH(tc.data(), type_curr, sizeof(int) * tiles), "copy")) return 1;
                for (int k = 0; k < tiles; ++k) types[(size_t)period * tiles + k] = (unsigned char)tc[k];
            }
            ++period;
        }
        int step = i, e1 = 1, e2 = 2;
        if (!launch(m, "kernel1_mix", grids_mix, blocks_mix,
                    {&eta1, &eta2_last, &eta2, &eta1_lap, &dfdeta1, &eta1_out, &heta1, &heta2, &heta1_lap, &hdfdeta1,
                     &heta1_out, &height, &hdxdy, &hone, &htwo, &hdtime, &hmobil, &hgrcoef, &type_curr, &step, &e1}) ||
            !launch(m, "kernel1_mix", grids_mix, blocks_mix,
                    {&eta2, &eta2_last, &eta1, &eta2_lap, &dfdeta2, &eta2_out, &heta2, &heta1, &heta2_lap, &hdfdeta2,
                     &heta2_out, &height, &hdxdy, &hone, &htwo, &hdtime, &hmobil, &hgrcoef, &type_curr, &step, &e2}) ||
            !ck(cuCtxSynchronize(), "sync"))
            return 1;
        std::swap(eta1, eta1_out);
        std::swap(eta2, eta2_out);
        std::swap(heta1, heta1_out);
        std::swap(heta2, heta2_out);
    }
    if (!t.stop(ms)) return 1;
    // end2end_mix.cu:118-120, for both fields
    if (!launch(m, "data_sychro_aftercomputation", grids_mix, blocks_mix, {&eta1, &heta1, &type_curr}) ||
        !launch(m, "data_sychro_aftercomputation", grids_mix, blocks_mix, {&eta2, &heta2, &type_curr}) ||
        !ck(cuCtxSynchronize(), "sync"))
        return 1;
    if (eta1_host && !ck(cuMemcpyDtoH(eta1_host, eta1, bytes), "copy")) return 1;
    if (eta2_host && !ck(cuMemcpyDtoH(eta2_host, eta2, bytes), "copy")) return 1;
    return 0;
}

}  // extern "C"

// The build's double constants (ref_consts, `count` of them).
static bool consts(RefModule *m, double *c, size_t count)
{
    CUdeviceptr p;
    size_t sz = 0;
    return ck(cuModuleGetGlobal(&p, &sz, m->mod, "ref_consts"), "ref_consts") && sz == sizeof(double) * count &&
           ck(cuMemcpyDtoH(c, p, sz), "ref_consts");
}

static bool set_threshold(RefModule *m, double thr)
{
    CUdeviceptr p;
    size_t sz = 0;
    return ck(cuModuleGetGlobal(&p, &sz, m->mod, "threshold"), "threshold") && sz == sizeof(double) &&
           ck(cuMemcpyHtoD(p, &thr, sizeof thr), "threshold");
}

extern "C" {

// snowflake/purehigh.cu:13-36 for `steps` steps: dataprepare_high (phi; T
// starts at 0), then per step kernel1_pure, kernel2_pure (in place) and a
// device synchronisation.  phi, T (host): the fields at the end; ms: the
// reference's elapsed time from step 5.
int refcuda_kob_pure(void *h, int steps, double *phi_host, double *t_host, float *ms)
{
    auto *m = static_cast<RefModule *>(h);
    if (!m || !current(m)) return 1;
    const int nx = m->dims[0], ny = m->dims[1], ux = m->dims[2], uy = m->dims[3];
    const size_t bytes = sizeof(double) * nx * ny;
    const unsigned tiles = (unsigned)((nx / ux) * (ny / uy));
    Buffers B;
    CUdeviceptr phi, phi_lap, tempr, tempr_lap, phidx, phidy, epsilon, epsilon_deri;
    for (CUdeviceptr *p : {&phi, &phi_lap, &tempr, &tempr_lap, &phidx, &phidy, &epsilon, &epsilon_deri})
        if (!B.get(*p, bytes)) return 1;
    const Dim blocks{(unsigned)ux, (unsigned)uy, 1}, grids{1, 1, tiles};
    if (!launch(m, "dataprepare_high", grids, blocks, {&phi}) || !ck(cuCtxSynchronize(), "sync")) return 1;
    Timer t;
    for (int i = 0; i < steps; ++i) {
        if (i == 5 && !t.start()) return 1;
        if (!launch(m, "kernel1_pure", grids, blocks,
                    {&phi, &phi_lap, &tempr, &tempr_lap, &phidx, &phidy, &epsilon, &epsilon_deri}) ||
            !launch(m, "kernel2_pure", grids, blocks,
                    {&phi, &phi_lap, &epsilon, &epsilon_deri, &phidx, &phidy, &tempr, &tempr_lap}) ||
            !ck(cuCtxSynchronize(), "sync"))
            return 1;
    }
    if (!t.stop(ms)) return 1;
    if (phi_host && !ck(cuMemcpyDtoH(phi_host, phi, bytes), "copy")) return 1;
    if (t_host && !ck(cuMemcpyDtoH(t_host, tempr, bytes), "copy")) return 1;
    return 0;
}

// snowflake/end2end_mix.cu:30-112 (AMSTENCIL) for `steps` steps at
// threshold `thr` with the cubin's monitor (`monitor`: 1 get_max_diff1 on
// phi, 2 get_max_diff2 against phi_old).  types, phi, T and ms as in
// refcuda_gg_mix (the fields gathered by data_sychro_aftercomputation).
int refcuda_kob_mix(void *h, int steps, double thr, int monitor, double *phi_host, double *t_host,
                    unsigned char *types, float *ms)
{
    auto *m = static_cast<RefModule *>(h);
    if (!m || !current(m) || (monitor != 1 && monitor != 2) || !set_threshold(m, thr)) return 1;
    const int nx = m->dims[0], ny = m->dims[1], ux = m->dims[2], uy = m->dims[3];
    const int ntx = nx / ux, nty = ny / uy, tiles = ntx * nty, uxd2 = ux / 2;
    const size_t n = (size_t)nx * ny, bytes = sizeof(double) * n, hbytes = sizeof(__half) * n;
    Buffers B;
    CUdeviceptr phi, phi_lap, tempr, tempr_lap, phidx, phidy, epsilon, epsilon_deri, phi_old;
    for (CUdeviceptr *p : {&phi, &phi_lap, &tempr, &tempr_lap, &phidx, &phidy, &epsilon, &epsilon_deri, &phi_old})
        if (!B.get(*p, bytes)) return 1;
    CUdeviceptr hphi, hphi_lap, htempr, htempr_lap, hphidx, hphidy, hepsilon, hepsilon_deri, type_new, type_old, max_diff;
    for (CUdeviceptr *p : {&hphi, &hphi_lap, &htempr, &htempr_lap, &hphidx, &hphidy, &hepsilon, &hepsilon_deri})
        if (!B.get(*p, hbytes)) return 1;
    if (!B.get(type_new, sizeof(int) * tiles) || !B.get(type_old, sizeof(int) * tiles) ||
        !B.get(max_diff, sizeof(double) * tiles))
        return 1;
    const Dim tile_grid{1, 1, (unsigned)tiles};
    if (!launch(m, "dataprepare_high", tile_grid, Dim{(unsigned)ux, (unsigned)uy, 1}, {&phi}) ||
        !ck(cuCtxSynchronize(), "sync") ||
        !launch(m, "dataprepare_half2", tile_grid, Dim{(unsigned)uxd2, (unsigned)uy, 1}, {&hphi}) ||
        !ck(cuCtxSynchronize(), "sync"))
        return 1;
    if (monitor == 2) {  // phi_old = (phi == 0), end2end_mix.cu:42-46
        std::vector<double> v(n);
        if (!ck(cuMemcpyDtoH(v.data(), phi, bytes), "copy")) return 1;
        for (double &x : v) x = x == 0 ? 1.0 : 0.0;
        if (!ck(cuMemcpyHtoD(phi_old, v.data(), bytes), "copy")) return 1;
    }
    double c[14];  // dxdy, dy*2, dx*2, theta0, aniso, delta, epsilonb, alpha, pi, gama, kappa, teq, dtime, tau
    if (!consts(m, c, 14)) return 1;
    __half2 hdxdy = __float2half2_rn(c[0]), hdym2 = __float2half2_rn(c[1]), hdxm2 = __float2half2_rn(c[2]),
            height = __float2half2_rn(8.0), htheta0 = __float2half2_rn(c[3]), haniso = __float2half2_rn(c[4]),
            hdelta = __float2half2_rn(c[5]), hone = __float2half2_rn(1.0), hepsilonb = __float2half2_rn(c[6]),
            halpha = __float2half2_rn(c[7]), hpi = __float2half2_rn(c[8]), hgama = __float2half2_rn(c[9]),
            hkappa = __float2half2_rn(c[10]), hzpf = __float2half2_rn(0.5), hteq = __float2half2_rn(c[11]),
            hdtime = __float2half2_rn(c[12]), htau = __float2half2_rn(c[13]);
    const Dim blocks_detect{(unsigned)(ntx > 32 ? 32 : ntx), (unsigned)(nty > 32 ? 32 : nty), 1};
    const Dim grids_detect{(unsigned)(ntx > 32 ? ntx / 32 : 1), (unsigned)(nty > 32 ? nty / 32 : 1), 1};
    const Dim sync_blocks{(unsigned)uxd2, (unsigned)uy, 1};
    const Dim blocks_mix{(unsigned)uxd2, (unsigned)uy, 1}, grids_mix{2, 1, (unsigned)tiles};
    Timer t;
    int period = 0;
    std::vector<int> tc(tiles);
    for (int i = 0; i < steps; ++i) {
        if (i == 5 && !t.start()) return 1;
        if (i % 10 == 0) {
            const bool ok = monitor == 1 ? launch(m, "get_max_diff1", grids_detect, blocks_detect, {&phi, &max_diff})
                                         : launch(m, "get_max_diff2", grids_detect, blocks_detect,
                                                  {&phi_old, &phi, &max_diff});
            if (!ok || !launch(m, "get_type", grids_detect, blocks_detect, {&max_diff, &type_old, &type_new}) ||
                !ck(cuCtxSynchronize(), "sync") ||
                !launch(m, "data_sychro_duringcomputation", tile_grid, sync_blocks,
                        {&phi, &tempr, &hphi, &htempr, &type_old, &type_new}) ||
                !ck(cuCtxSynchronize(), "sync"))
                return 1;
            if (types) {
                if (!ck(cuMemcpyDtoH(tc.data(), type_new, sizeof(int) * tiles), "copy")) return 1;
                for (int k = 0; k < tiles; ++k) types[(size_t)period * tiles + k] = (unsigned char)tc[k];
            }
            ++period;
        }
        int step = i;
        if (!launch(m, "kernel1_mix", grids_mix, blocks_mix,
                    {&phi, &phi_old, &phi_lap, &epsilon, &epsilon_deri, &phidx, &phidy, &tempr, &tempr_lap, &hphi,
                     &hphi_lap, &htempr, &htempr_lap, &hphidx, &hphidy, &hepsilon, &hepsilon_deri, &hdxdy, &htheta0,
                     &haniso, &hone, &hdxm2, &hdym2, &hdelta, &hepsilonb, &height, &type_new, &step}) ||
            !launch(m, "mix_kernel2", grids_mix, blocks_mix,
                    {&phi, &phi_lap, &epsilon, &epsilon_deri, &phidx, &phidy, &tempr, &tempr_lap, &hphi, &hphi_lap,
                     &hepsilon, &hepsilon_deri, &hphidx, &hphidy, &htempr, &htempr_lap, &hdym2, &hdxm2, &hgama,
                     &hteq, &halpha, &hpi, &hone, &hzpf, &hdtime, &htau, &hkappa, &type_new, &step}) ||
            !ck(cuCtxSynchronize(), "sync"))
            return 1;
    }
    if (!t.stop(ms)) return 1;
    // end2end_mix.cu:117-120, for both fields
    if (!launch(m, "data_sychro_aftercomputation", grids_mix, blocks_mix, {&phi, &hphi, &type_new}) ||
        !launch(m, "data_sychro_aftercomputation", grids_mix, blocks_mix, {&tempr, &htempr, &type_new}) ||
        !ck(cuCtxSynchronize(), "sync"))
        return 1;
    if (phi_host && !ck(cuMemcpyDtoH(phi_host, phi, bytes), "copy")) return 1;
    if (t_host && !ck(cuMemcpyDtoH(t_host, tempr, bytes), "copy")) return 1;
    return 0;
}

}  // extern "C"

extern "C" {

// sintering/main.cu:136-147 (PURE) for `steps` steps from the caller's
// state: con1_pure, con2_pure, phi1_pure, phi2_pure, each followed by a device
// synchronisation, then the swap.  c, e1, e2 (host, dimX*dimY): the initial
// state in, the fields at the end out; ms: the elapsed time from step 5.
int refcuda_sint_pure(void *h, int steps, double *c_host, double *e1_host, double *e2_host, float *ms)
{
    auto *m = static_cast<RefModule *>(h);
    if (!m || !current(m)) return 1;
    const int nx = m->dims[0], ny = m->dims[1], ux = m->dims[2], uy = m->dims[3];
    const size_t bytes = sizeof(double) * nx * ny;
    const unsigned tiles = (unsigned)((nx / ux) * (ny / uy));
    Buffers B;
    CUdeviceptr con, eta1, eta2, eta1_out, eta2_out, con_lap, eta1_lap, eta2_lap, dummy, dummy_lap, dfdcon, dfdeta1,
        dfdeta2;
    for (CUdeviceptr *p : {&con, &eta1, &eta2, &eta1_out, &eta2_out, &con_lap, &eta1_lap, &eta2_lap, &dummy, &dummy_lap,
                           &dfdcon, &dfdeta1, &dfdeta2})
        if (!B.get(*p, bytes)) return 1;
    if (!ck(cuMemcpyHtoD(con, c_host, bytes), "copy") || !ck(cuMemcpyHtoD(eta1, e1_host, bytes), "copy") ||
        !ck(cuMemcpyHtoD(eta2, e2_host, bytes), "copy"))
        return 1;
    const Dim blocks{(unsigned)ux, (unsigned)uy, 1}, grids{1, 1, tiles};
    Timer t;
    for (int i = 0; i < steps; ++i) {
        if (i == 5 && !t.start()) return 1;
        int step = i;
        if (!launch(m, "con1_pure", grids, blocks, {&con, &con_lap, &eta1, &eta2, &dfdcon, &dummy, &step}) ||
            !ck(cuCtxSynchronize(), "sync") ||
            !launch(m, "con2_pure", grids, blocks, {&dummy, &dummy_lap, &con, &eta1, &eta2, &step}) ||
            !ck(cuCtxSynchronize(), "sync") ||
            !launch(m, "phi1_pure", grids, blocks, {&eta1, &eta1_out, &eta2, &eta1_lap, &dfdeta1, &con, &step}) ||
            !ck(cuCtxSynchronize(), "sync") ||
            !launch(m, "phi2_pure", grids, blocks, {&eta2, &eta2_out, &eta1, &eta2_lap, &dfdeta2, &con, &step}) ||
            !ck(cuCtxSynchronize(), "sync"))
            return 1;
        std::swap(eta1, eta1_out);
        std::swap(eta2, eta2_out);
    }
    if (!t.stop(ms)) return 1;
    return !(ck(cuMemcpyDtoH(c_host, con, bytes), "copy") && ck(cuMemcpyDtoH(e1_host, eta1, bytes), "copy") &&
             ck(cuMemcpyDtoH(e2_host, eta2, bytes), "copy"));
}

// sintering/main.cu:66-206 (AMSTENCIL) for `steps` steps from the caller's
// state at threshold `thr` (`monitor`: 1 get_max_diff1 on c, 2 get_max_diff2
// against con_old).  types: [ceil(steps/10)][tiles] uint8 (1 half2, 2 high);
// c, e1, e2 in/out as in refcuda_sint_pure (the half tiles gathered by
// data_sychro_aftercomputation); ms: the elapsed time from step 5.
int refcuda_sint_mix(void *h, int steps, double thr, int monitor, double *c_host, double *e1_host, double *e2_host,
                     unsigned char *types, float *ms)
{
    auto *m = static_cast<RefModule *>(h);
    if (!m || !current(m) || (monitor != 1 && monitor != 2)) return 1;
    const int nx = m->dims[0], ny = m->dims[1], ux = m->dims[2], uy = m->dims[3];
    const int ntx = nx / ux, nty = ny / uy, tiles = ntx * nty, uxd2 = ux / 2;
    const size_t n = (size_t)nx * ny, bytes = sizeof(double) * n, hbytes = sizeof(__half) * n;
    Buffers B;
    CUdeviceptr con, eta1, eta2, eta1_out, eta2_out, con_lap, eta1_lap, eta2_lap, dummy, dummy_lap, dfdcon, dfdeta1,
        dfdeta2, con_old;
    for (CUdeviceptr *p : {&con, &eta1, &eta2, &eta1_out, &eta2_out, &con_lap, &eta1_lap, &eta2_lap, &dummy, &dummy_lap,
                           &dfdcon, &dfdeta1, &dfdeta2, &con_old})
        if (!B.get(*p, bytes)) return 1;
    CUdeviceptr hcon, heta1, heta2, heta1_out, heta2_out, hcon_lap, heta1_lap, heta2_lap, hdummy, hdummy_lap, hdfdcon,
        hdfdeta1, hdfdeta2, type_con, type_old, max_diff;
    for (CUdeviceptr *p : {&hcon, &heta1, &heta2, &heta1_out, &heta2_out, &hcon_lap, &heta1_lap, &heta2_lap, &hdummy,
                           &hdummy_lap, &hdfdcon, &hdfdeta1, &hdfdeta2})
        if (!B.get(*p, hbytes)) return 1;
    if (!B.get(type_con, sizeof(int) * tiles) || !B.get(type_old, sizeof(int) * tiles) ||
        !B.get(max_diff, sizeof(double) * tiles))
        return 1;
    {
        std::vector<double> old(n);
        for (size_t k = 0; k < n; ++k) old[k] = c_host[k] == 0 ? 1.0 : 0.0;  // main.cu:61-64
        if (!ck(cuMemcpyHtoD(con, c_host, bytes), "copy") || !ck(cuMemcpyHtoD(eta1, e1_host, bytes), "copy") ||
            !ck(cuMemcpyHtoD(eta2, e2_host, bytes), "copy") || !ck(cuMemcpyHtoD(con_old, old.data(), bytes), "copy"))
            return 1;
    }
    const Dim blocks_dp{32, 32, 1}, grids_dp{(unsigned)(nx / 32 / 2), (unsigned)(ny / 32), 1};
    if (!launch(m, "dataprepare", grids_dp, blocks_dp, {&con, &hcon}) ||
        !launch(m, "dataprepare", grids_dp, blocks_dp, {&eta1, &heta1}) ||
        !launch(m, "dataprepare", grids_dp, blocks_dp, {&eta2, &heta2}) || !ck(cuCtxSynchronize(), "sync"))
        return 1;
    double c[9];  // coefm, coefk, coefl, dvol, dvap, dsur, dgrb, dxdy, dtime
    if (!consts(m, c, 9)) return 1;
    auto h2 = [](double v) { return __floats2half2_rn(v, v); };  // lowprecision2highprecision, sintering/tools.h:122
    __half2 hcoefm = h2(c[0]), hcoefk = h2(c[1]), hcoefl = h2(c[2]), hdvol = h2(c[3]), hdvap = h2(c[4]),
            hdsur = h2(c[5]), hdgrb = h2(c[6]), hdxdy = h2(c[7]), hdtime = h2(c[8]), hcf = h2(4.0), hzpfive = h2(0.5),
            hone = h2(1.0), htwo = h2(2.0), hfour = h2(4.0), hsix = h2(6.0), hten = h2(10.0), htwelve = h2(12.0),
            hfifteen = h2(15.0), hthirtytwo = h2(32.0), highbound = h2(1), lowbound = h2(0.0);
    const Dim blocks{(unsigned)uxd2, (unsigned)uy, 1}, grids{2, 1, (unsigned)tiles};
    const Dim blocks_detect{(unsigned)(ntx > 32 ? 32 : ntx), (unsigned)(nty > 32 ? 32 : nty), 1};
    const Dim grids_detect{(unsigned)(ntx > 32 ? ntx / 32 : 1), (unsigned)(nty > 32 ? nty / 32 : 1), 1};
    const Dim sync_blocks{(unsigned)uxd2, (unsigned)uy, 1}, sync_grids{1, 1, (unsigned)tiles};
    Timer t;
    int period = 0;
    std::vector<int> tc(tiles);
    for (int i = 0; i < steps; ++i) {
        if (i == 5 && !t.start()) return 1;
        if (i % 10 == 0) {
            const bool ok = monitor == 1 ? launch(m, "get_max_diff1", grids_detect, blocks_detect, {&con, &max_diff})
                                         : launch(m, "get_max_diff2", grids_detect, blocks_detect,
                                                  {&con_old, &con, &max_diff});
            if (!ok ||
                !launch(m, "ref_get_type_rt", grids_detect, blocks_detect, {&max_diff, &type_old, &type_con, &thr}) ||
                !ck(cuCtxSynchronize(), "sync") ||
                !launch(m, "data_sychro_duringcomputation", sync_grids, sync_blocks,
                        {&con, &eta1, &eta2, &hcon, &heta1, &heta2, &type_old, &type_con}) ||
                !ck(cuCtxSynchronize(), "sync"))
                return 1;
            if (types) {
                if (!ck(cuMemcpyDtoH(tc.data(), type_con, sizeof(int) * tiles), "copy")) return 1;
                for (int k = 0; k < tiles; ++k) types[(size_t)period * tiles + k] = (unsigned char)tc[k];
            }
            ++period;
        }
        int step = i;
        if (!launch(m, "con1_mix", grids, blocks,
                    {&type_con, &con, &con_old, &con_lap, &eta1, &eta2, &dfdcon, &dummy, &hcon, &hcon_lap, &heta1,
                     &heta2, &hdfdcon, &hdummy, &hcf, &hdxdy, &hsix, &hzpfive, &hone, &htwo, &hfour, &hthirtytwo,
                     &hcoefm, &step}) ||
            !ck(cuCtxSynchronize(), "sync") ||
            !launch(m, "con2_mix", grids, blocks,
                    {&type_con, &dummy, &dummy_lap, &con, &eta1, &eta2, &hdummy, &hdummy_lap, &hcon, &heta1, &heta2,
                     &hcf, &hdxdy, &hone, &htwo, &hsix, &hten, &hfifteen, &hdgrb, &hdsur, &hdtime, &hdvap, &hdvol,
                     &highbound, &lowbound, &step}) ||
            !ck(cuCtxSynchronize(), "sync") ||
            !launch(m, "phi1_mix", grids, blocks,
                    {&type_con, &eta1, &eta1_out, &eta2, &eta1_lap, &dfdeta1, &con, &heta1, &heta1_out, &heta2,
                     &heta1_lap, &hdfdeta1, &hcon, &hcf, &hdxdy, &hzpfive, &hone, &htwo, &htwelve, &hdtime, &hcoefl,
                     &hcoefk, &highbound, &lowbound, &step}) ||
            !ck(cuCtxSynchronize(), "sync") ||
            !launch(m, "phi2_mix", grids, blocks,
                    {&type_con, &eta2, &eta2_out, &eta1, &eta2_lap, &dfdeta2, &con, &heta2, &heta2_out, &heta1,
                     &heta2_lap, &hdfdeta2, &hcon, &hcf, &hdxdy, &hzpfive, &hone, &htwo, &htwelve, &hdtime, &hcoefl,
                     &hcoefk, &highbound, &lowbound, &step}) ||
            !ck(cuCtxSynchronize(), "sync"))
            return 1;
        std::swap(eta1, eta1_out);
        std::swap(eta2, eta2_out);
        std::swap(heta1, heta1_out);
        std::swap(heta2, heta2_out);
    }
    if (!t.stop(ms)) return 1;
    if (!launch(m, "data_sychro_aftercomputation", grids_dp, blocks_dp, {&con, &hcon, &type_con}) ||
        !launch(m, "data_sychro_aftercomputation", grids_dp, blocks_dp, {&eta1, &heta1, &type_con}) ||
        !launch(m, "data_sychro_aftercomputation", grids_dp, blocks_dp, {&eta2, &heta2, &type_con}) ||
        !ck(cuCtxSynchronize(), "sync"))
        return 1;
    return !(ck(cuMemcpyDtoH(c_host, con, bytes), "copy") && ck(cuMemcpyDtoH(e1_host, eta1, bytes), "copy") &&
             ck(cuMemcpyDtoH(e2_host, eta2, bytes), "copy"));
}

}  // extern "C"

extern "C" {

// graingrowth/purelow.cu:3-47 (HALF2) for `steps` steps: dataprepare_half2,
// then per step kernel1_lowpure for eta1 and for eta2, a device
// synchronisation and the swap.  eta1, eta2 (host, dimX*dimY/2 half2 pairs as
// 32-bit words): the fields at the end; ms: the elapsed time from step 5.
int refcuda_gg_purelow(void *h, int steps, uint32_t *eta1_host, uint32_t *eta2_host, float *ms)
{
    auto *m = static_cast<RefModule *>(h);
    if (!m || !current(m)) return 1;
    const int nx = m->dims[0], ny = m->dims[1], ux = m->dims[2], uy = m->dims[3];
    const size_t hbytes = sizeof(__half) * nx * ny;
    const unsigned tiles = (unsigned)((nx / ux) * (ny / uy));
    Buffers B;
    CUdeviceptr eta1, eta2, eta1_out, eta2_out, eta1_lap, eta2_lap, dfdeta1, dfdeta2;
    for (CUdeviceptr *p : {&eta1, &eta2, &eta1_out, &eta2_out, &eta1_lap, &eta2_lap, &dfdeta1, &dfdeta2})
        if (!B.get(*p, hbytes)) return 1;
    const Dim blocks{(unsigned)(ux / 2), (unsigned)uy, 1}, grids{1, 1, tiles};
    if (!launch(m, "dataprepare_half2", grids, blocks, {&eta1, &eta2}) || !ck(cuCtxSynchronize(), "sync")) return 1;
    double c[4];  // mobil, grcoef, dxdy, dtime
    if (!consts(m, c, 4)) return 1;
    __half2 hmobil = __float2half2_rn(c[0]), hgrcoef = __float2half2_rn(c[1]), hdxdy = __float2half2_rn(c[2]),
            hdtime = __float2half2_rn(c[3]), height = __float2half2_rn(8.0), hone = __float2half2_rn(1.0),
            htwo = __float2half2_rn(2.0);
    Timer t;
    for (int i = 0; i < steps; ++i) {
        if (i == 5 && !t.start()) return 1;
        if (!launch(m, "kernel1_lowpure", grids, blocks,
                    {&eta1, &eta2, &eta1_lap, &dfdeta1, &eta1_out, &hone, &htwo, &height, &hdtime, &hmobil, &hgrcoef,
                     &hdxdy}) ||
            !launch(m, "kernel1_lowpure", grids, blocks,
                    {&eta2, &eta1, &eta2_lap, &dfdeta2, &eta2_out, &hone, &htwo, &height, &hdtime, &hmobil, &hgrcoef,
                     &hdxdy}) ||
            !ck(cuCtxSynchronize(), "sync"))
            return 1;
        std::swap(eta1, eta1_out);
        std::swap(eta2, eta2_out);
    }
    if (!t.stop(ms)) return 1;
    return !(ck(cuMemcpyDtoH(eta1_host, eta1, hbytes), "copy") && ck(cuMemcpyDtoH(eta2_host, eta2, hbytes), "copy"));
}

// snowflake/purelow.cu:3-66 (HALF2) for `steps` steps: dataprepare_half2
// (phi; T starts at 0), then per step kernel1_purelow, kernel2_purelow (in
// place) and a device synchronisation.  phi, T (host, half2 pairs as 32-bit
// words): the fields at the end; ms: the elapsed time from step 5.
int refcuda_kob_purelow(void *h, int steps, uint32_t *phi_host, uint32_t *t_host, float *ms)
{
    auto *m = static_cast<RefModule *>(h);
    if (!m || !current(m)) return 1;
    const int nx = m->dims[0], ny = m->dims[1], ux = m->dims[2], uy = m->dims[3];
    const size_t hbytes = sizeof(__half) * nx * ny;
    const unsigned tiles = (unsigned)((nx / ux) * (ny / uy));
    Buffers B;
    CUdeviceptr phi, phi_lap, tempr, tempr_lap, phidx, phidy, epsilon, epsilon_deri;
    for (CUdeviceptr *p : {&phi, &phi_lap, &tempr, &tempr_lap, &phidx, &phidy, &epsilon, &epsilon_deri})
        if (!B.get(*p, hbytes)) return 1;
    const Dim blocks{(unsigned)(ux / 2), (unsigned)uy, 1}, grids{1, 1, tiles};
    if (!launch(m, "dataprepare_half2", grids, blocks, {&phi}) || !ck(cuCtxSynchronize(), "sync")) return 1;
    double c[14];  // dxdy, dy*2, dx*2, theta0, aniso, delta, epsilonb, alpha, pi, gama, kappa, teq, dtime, tau
    if (!consts(m, c, 14)) return 1;
    __half2 hdxdy = __float2half2_rn(c[0]), hdym2 = __float2half2_rn(c[1]), hdxm2 = __float2half2_rn(c[2]),
            height = __float2half2_rn(8.0), htheta0 = __float2half2_rn(c[3]), haniso = __float2half2_rn(c[4]),
            hdelta = __float2half2_rn(c[5]), hone = __float2half2_rn(1.0), hepsilonb = __float2half2_rn(c[6]),
            halpha = __float2half2_rn(c[7]), hpi = __float2half2_rn(c[8]), hgama = __float2half2_rn(c[9]),
            hkappa = __float2half2_rn(c[10]), hzpf = __float2half2_rn(0.5), hteq = __float2half2_rn(c[11]),
            hdtime = __float2half2_rn(c[12]), htau = __float2half2_rn(c[13]);
    Timer t;
    for (int i = 0; i < steps; ++i) {
        if (i == 5 && !t.start()) return 1;
        if (!launch(m, "kernel1_purelow", grids, blocks,
                    {&phi, &phi_lap, &tempr, &tempr_lap, &phidx, &phidy, &epsilon, &epsilon_deri, &hdxdy, &htheta0,
                     &haniso, &hone, &hdxm2, &hdym2, &hdelta, &hepsilonb, &height}) ||
            !launch(m, "kernel2_purelow", grids, blocks,
                    {&phi, &phi_lap, &epsilon, &epsilon_deri, &phidx, &phidy, &tempr, &tempr_lap, &hdym2, &hdxm2,
                     &hgama, &hteq, &halpha, &hpi, &hone, &hzpf, &hdtime, &htau, &hkappa}) ||
            !ck(cuCtxSynchronize(), "sync"))
            return 1;
    }
    if (!t.stop(ms)) return 1;
    return !(ck(cuMemcpyDtoH(phi_host, phi, hbytes), "copy") && ck(cuMemcpyDtoH(t_host, tempr, hbytes), "copy"));
}

}  // extern "C"
