// Drop-in SOAP_resolution: the argv / file contract of SOAP_resolution.cu:318-440 on
// top of libsoapgb (soapgb_lower_resolution, all phases of a type in one call).
//
// argv: n_phase N sigma_v raw_dir spec_dir no_block no_thread file_prefix quiet_prefix
// reads:  <quiet_prefix>_{quiet_sun,SED_quiet_sun}_spec.bin, <quiet_prefix>_quiet_sun_wave.bin,
//         raw_dir/<prefix>_Spec_{tot,flux,bconv}_<i>_.bin
// writes: spec_dir/<prefix>_lower_spec_{tot,flux,bconv}_<i>_.bin
#include "tool_common.h"

int main(int argc, char *argv[]) {
    tool::Timer timer;
    tool::need_args(argc, 9, "n_phase N sigma_v raw_dir spec_dir no_block no_thread file_prefix quiet_prefix");
    int npsi = std::atoi(argv[1]);
    int n = std::atoi(argv[2]);
    double sigma_v = std::atof(argv[3]);
    std::string raw_dir = argv[4];
    std::string spec_dir = argv[5];
    int no_block = std::atoi(argv[6]);
    int no_thread = std::atoi(argv[7]);
    std::string prefix = argv[8];
    std::string quiet_prefix = argv[9];
    long long n_eff = (long long)no_block * no_thread;
    if (npsi < 0 || n < 3 || n_eff < 2 || n_eff > n)
        tool::die("inconsistent sizes: N=" + std::to_string(n) + " no_block*no_thread=" + std::to_string(n_eff));
    int form = tool::form_from_env();
    // files hold n_eff values; the n-long buffers keep a zero tail
    std::vector<double> q_norm = tool::read_f64(quiet_prefix + "_quiet_sun_spec.bin", n_eff, n);
    std::vector<double> q_sed = tool::read_f64(quiet_prefix + "_SED_quiet_sun_spec.bin", n_eff, n);
    std::vector<double> wave = tool::read_f64(quiet_prefix + "_quiet_sun_wave.bin", n_eff, n);
    soapgb_ctx *ctx = tool::open_ctx();
    const char *types[3] = {"tot", "flux", "bconv"};
    // tot and flux use the SED quiet spectrum, bconv the normalised one (SOAP_resolution.cu:414-416)
    for (int t = 0; t < 3; ++t) {
        std::vector<double> spec((size_t)n * (npsi > 0 ? npsi : 1), 0.0);
        for (int p = 0; p < npsi; ++p) {
            std::vector<double> v = tool::read_f64(
                raw_dir + prefix + "_Spec_" + types[t] + "_" + std::to_string(p) + "_.bin", n_eff);
            std::copy(v.begin(), v.end(), spec.begin() + (size_t)n * p);
        }
        std::vector<double> low((size_t)n_eff * (npsi > 0 ? npsi : 1));
        const double *base = (t == 2) ? q_norm.data() : q_sed.data();
        // SOAP_resolution.cu:80,86: step 0.005 in both the multiplier and the exponent
        tool::check(ctx,
                    soapgb_lower_resolution(ctx, form, n, (int)n_eff, npsi, wave.data(), base, spec.data(), sigma_v,
                                            50.0, 0.005, 0.005, -60000.0, SOAPGB_HOST, low.data(), nullptr),
                    "lower resolution");
        for (int p = 0; p < npsi; ++p)
            tool::write_bin(spec_dir + prefix + "_lower_spec_" + types[t] + "_" + std::to_string(p) + "_.bin",
                            low.data() + (size_t)n_eff * p, n_eff);
    }
    for (int p = 0; p < npsi; ++p) std::printf("PHASE = %d over %d\n", p, npsi);
    soapgb_ctx_destroy(ctx);
    timer.report();
    return 0;
}
