// amps_driver -- the reference's driver programs over the libamps C ABI.
//
// One executable; the program it acts as comes from the name it is invoked
// under (the build links these names to it) or from the first argument:
//
//   snowflake_purehigh  <runIdx> <csvPath>   snowflake/purehigh.cu:3-66
//   snowflake_end2end_mix <runIdx> <csvPath> snowflake/end2end_mix.cu:3-147
//   snowflake_purelow                        snowflake/purelow.cu:3-82
//   graingrowth_purehigh / _end2end_mix / _purelow   graingrowth/*.cu (same CLI)
//   sintering_main <paraIdx> <datatype>      sintering/main.cu:5-635
//
// As in the reference, every program writes time_tmp.csv (device time in ms
// from step 5 to the end), the snowflake/grain-growth programs dump phi /
// eta2 to <csvPath> when runIdx is "4", purelow writes half2result.csv
// (halfresult.csv with --half), and sintering_main writes c under
// ./result/end2end/<datatype>/<strategy>/[monitor<k>/]para<p>/.  The settings
// the reference's sweep scripts write into its headers are flags here:
//   --para N (1..5, default 5: the shipped #include of paras/para5.h)
//   --dtype double|float   --timesteps N (500)   --threshold X (0.99)
//   --monitor 1|2 (2)      --strategy pure|amstencil|gram1|gram2   --ratio R (1.0)
#include "../../include/amps.h"

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace {

struct Opts {
    std::string prog;
    std::vector<std::string> pos;
    int para = 5, timesteps = 500, monitor = 2;
    std::string dtype = "double", strategy;
    double threshold = 0.99, ratio = 1.0;
    bool half = false;
};

int die(const char *what, amps_handle *h)
{
    fprintf(stderr, "%s: %s\n", what, amps_last_error(h));
    return 1;
}

// snowflake/tools.h:4-23: header ",0,1,...,X-1", then "y,v0,...,vX-1"
template <typename T> void writetocsv(const std::string &path, const T *data, int X, int Y)
{
    std::ofstream f(path);
    f << ",";
    for (int x = 0; x < X; ++x) f << x << (x == X - 1 ? "\n" : ",");
    for (int y = 0; y < Y; ++y) {
        f << y << ",";
        for (int x = 0; x < X; ++x) f << data[(size_t)y * X + x] << (x == X - 1 ? "\n" : ",");
    }
}

void mkdirs(const std::string &path)
{
    for (size_t i = 1; i <= path.size(); ++i)
        if (i == path.size() || path[i] == '/') mkdir(path.substr(0, i).c_str(), 0777);
}

// Run the time loop; returns device ms from step 5 to the end (the reference's window).
int timed_run(amps_handle *h, int steps, float *ms)
{
    cudaStream_t s;
    if (cudaStreamCreate(&s) != cudaSuccess) return AMPS_ERR_CUDA;
    if (int r = amps_set_stream(h, s)) return r;
    *ms = 0.f;
    const int warm = steps < 5 ? steps : 5;
    if (int r = amps_run(h, warm)) return r;
    if (steps > 5) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, s);
        if (int r = amps_run(h, steps - 5)) return r;
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        cudaEventElapsedTime(ms, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
    int r = amps_synchronize(h);
    amps_set_stream(h, nullptr);
    cudaStreamDestroy(s);
    return r;
}

int configure(const Opts &o, int model, int mode, amps_params *p)
{
    if (amps_preset(model, o.para, p)) return 1;
    p->mode = mode;
    p->high_tier = o.dtype == "float" ? AMPS_TIER_FP32 : AMPS_TIER_FP64;
    p->monitor = o.monitor;
    p->thr_lo = p->thr_hi = o.threshold;
    p->gram_ratio = o.ratio;
    return 0;
}

int run_app(const Opts &o, int model, const std::string &kind)
{
    amps_params p;
    int mode = kind == "purehigh" ? AMPS_PUREHIGH : kind == "purelow" ? AMPS_PURELOW : AMPS_END2END_MIX;
    if (kind == "end2end_mix" && o.strategy == "gram1") mode = AMPS_GRAM1;
    if (kind == "end2end_mix" && o.strategy == "gram2") mode = AMPS_GRAM2;
    if (configure(o, model, mode, &p)) return die("parameters", nullptr);
    amps_handle *h = nullptr;
    if (amps_create(&p, &h)) return die("amps_create", nullptr);
    if (amps_init(h, AMPS_INIT_REFERENCE)) return die("amps_init", h);
    float ms = 0.f;
    if (timed_run(h, o.timesteps, &ms)) return die("amps_run", h);
    std::ofstream("time_tmp.csv") << ms;
    // the monitored field: phi (snowflake/purehigh.cu:50), eta2 (graingrowth/purehigh.cu:52)
    const int field = model == AMPS_GRAINGROWTH ? 1 : 0;
    std::vector<double> f((size_t)p.nx * p.ny);
    if (kind == "purelow") {
        // snowflake/purelow.cu:66-71: float dump of the half state
        std::vector<float> ff(f.size());
        if (amps_get_field(h, field, ff.data(), AMPS_F32, 0)) return die("amps_get_field", h);
        const char *name = o.half ? "halfresult.csv" : "half2result.csv";
        writetocsv(name, ff.data(), p.nx, p.ny);
        printf("%s\n", name);
    } else if (o.pos.size() >= 2 && o.pos[0] == "4") {
        if (p.high_tier == AMPS_TIER_FP32) {
            std::vector<float> ff(f.size());
            if (amps_get_field(h, field, ff.data(), AMPS_F32, 0)) return die("amps_get_field", h);
            writetocsv(o.pos[1], ff.data(), p.nx, p.ny);
        } else {
            if (amps_get_field(h, field, f.data(), AMPS_F64, 0)) return die("amps_get_field", h);
            writetocsv(o.pos[1], f.data(), p.nx, p.ny);
        }
    }
    amps_destroy(h);
    return 0;
}

// sintering/main.cu: argv[1] = para index, argv[2] = datatype; result tree of :445-520
int run_sintering(Opts o)
{
    if (o.pos.size() < 2) {
        fprintf(stderr, "usage: sintering_main <paraIdx> <datatype> [--strategy pure|amstencil|gram1|gram2] ...\n");
        return 2;
    }
    o.para = atoi(o.pos[0].c_str());
    o.dtype = o.pos[1];
    const std::string strat = o.strategy.empty() ? "pure" : o.strategy;
    const int mode = strat == "pure" ? AMPS_PUREHIGH : strat == "gram1" ? AMPS_GRAM1 : strat == "gram2" ? AMPS_GRAM2
                                                                                                  : AMPS_END2END_MIX;
    amps_params p;
    if (configure(o, AMPS_SINTERING, mode, &p)) return die("parameters", nullptr);
    amps_handle *h = nullptr;
    if (amps_create(&p, &h)) return die("amps_create", nullptr);
    if (amps_init(h, AMPS_INIT_REFERENCE)) return die("amps_init", h);
    float ms = 0.f;
    if (timed_run(h, o.timesteps, &ms)) return die("amps_run", h);
    std::ofstream("time_tmp.csv") << ms;
    std::string dir = "./result/end2end/" + o.dtype + "/" + (strat == "amstencil" ? "amstencil" : strat) + "/";
    std::string name = std::to_string(o.timesteps);
    if (strat == "amstencil") {
        dir += "monitor" + std::to_string(o.monitor) + "/";
        std::ostringstream t;
        if (o.monitor == 1) t << std::to_string(o.threshold);  // to_string(threshold), Monitor1
        else t << o.threshold;                                  // ostream formatting, Monitor2
        name += "_" + t.str();
    } else if (strat == "gram1" || strat == "gram2") {
        name += "_" + std::to_string(o.ratio);
    }
    dir += "para" + o.pos[0] + "/";
    mkdirs(dir);
    std::vector<double> c((size_t)p.nx * p.ny);
    if (amps_get_field(h, 0, c.data(), AMPS_F64, 0)) return die("amps_get_field", h);
    writetocsv(dir + name + ".csv", c.data(), p.nx, p.ny);
    amps_destroy(h);
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    Opts o;
    std::string self = argv[0];
    const size_t sl = self.rfind('/');
    o.prog = sl == std::string::npos ? self : self.substr(sl + 1);
    int i = 1;
    if (o.prog == "amps_driver") {
        if (argc < 2) {
            fprintf(stderr, "usage: amps_driver <snowflake|graingrowth>_<purehigh|purelow|end2end_mix> | sintering_main ...\n");
            return 2;
        }
        o.prog = argv[1];
        i = 2;
    }
    for (; i < argc; ++i) {
        std::string a = argv[i];
        auto val = [&]() { return i + 1 < argc ? std::string(argv[++i]) : std::string(); };
        if (a == "--para") o.para = atoi(val().c_str());
        else if (a == "--dtype") o.dtype = val();
        else if (a == "--timesteps") o.timesteps = atoi(val().c_str());
        else if (a == "--threshold") o.threshold = atof(val().c_str());
        else if (a == "--monitor") o.monitor = atoi(val().c_str());
        else if (a == "--strategy") o.strategy = val();
        else if (a == "--ratio") o.ratio = atof(val().c_str());
        else if (a == "--half") o.half = true;
        else o.pos.push_back(a);
    }
    if (o.prog == "sintering_main") return run_sintering(o);
    const size_t us = o.prog.find('_');
    if (us == std::string::npos) {
        fprintf(stderr, "unknown program %s\n", o.prog.c_str());
        return 2;
    }
    const std::string app = o.prog.substr(0, us), kind = o.prog.substr(us + 1);
    const int model = app == "snowflake" ? AMPS_KOBAYASHI : app == "graingrowth" ? AMPS_GRAINGROWTH : -1;
    if (model < 0 || (kind != "purehigh" && kind != "purelow" && kind != "end2end_mix")) {
        fprintf(stderr, "unknown program %s\n", o.prog.c_str());
        return 2;
    }
    // end2end_mix without --strategy is AMSTENCIL (snowflake/paras/total.h:25)
    return run_app(o, model, kind);
}
