// Drop-in SOAP_initialize: the argv / file contract of SOAP_initialize.cu:508-610
// on top of libsoapgb (soapgb_disk_maps, soapgb_quiet_disk, soapgb_lower_resolution).
//
// argv: N P W_ratio I R_km u1 u2 G sigma_v step step_median window no_block
//       no_thread cube.bin out_prefix n_mu mu_bounds.bin wave.bin LB0 LB1 LB2 LB3
// writes: <prefix>{mu,delta,limb,region,LB}_map.bin, <prefix>_quiet_sun_spec.bin,
//         <prefix>_quiet_sun_wave.bin, <prefix>_quiet_sun_lower_spec.bin
#include "tool_common.h"

int main(int argc, char *argv[]) {
    tool::Timer timer;
    tool::need_args(argc, 23,
                    "N P W_ratio I R_km u1 u2 G sigma_v step step_median window no_block no_thread cube.bin "
                    "out_prefix n_mu mu_bounds.bin wave.bin LB0 LB1 LB2 LB3");
    int n = std::atoi(argv[1]);
    soapgb_star st;
    st.period = std::atof(argv[2]);
    st.omega_ratio = std::atof(argv[3]);
    st.incl = std::atof(argv[4]);
    st.radius_km = std::atof(argv[5]);
    st.u1 = std::atof(argv[6]);
    st.u2 = std::atof(argv[7]);
    st.grid = std::atoi(argv[8]);
    double sigma_v = std::atof(argv[9]);
    double step = std::atof(argv[10]);
    double step_median = std::atof(argv[11]);
    double window = std::atof(argv[12]);
    int no_block = std::atoi(argv[13]);
    int no_thread = std::atoi(argv[14]);
    std::string cube_name = argv[15];
    std::string prefix = argv[16];
    int n_mu = std::atoi(argv[17]);
    std::string mu_name = argv[18];
    std::string wave_name = argv[19];
    for (int q = 0; q < 4; ++q) st.lb[q] = std::atof(argv[20 + q]);
    long long n_eff = (long long)no_block * no_thread;
    if (n < 3 || n_mu < 1 || st.grid < 1 || n_eff < 2 || n_eff > n)
        tool::die("inconsistent sizes: N=" + std::to_string(n) + " no_block*no_thread=" + std::to_string(n_eff));
    int form = tool::form_from_env();

    std::vector<double> cube = tool::read_f64(cube_name, (size_t)n * n_mu);
    std::vector<double> wave = tool::read_f64(wave_name, n);
    std::vector<double> mu_b = n_mu > 1 ? tool::read_f64(mu_name, n_mu - 1) : std::vector<double>(1, 0.0);

    soapgb_ctx *ctx = tool::open_ctx();
    long long gm = (long long)st.grid * st.grid;
    std::vector<double> delta(gm), limb(gm), mu(gm), lb(gm);
    std::vector<int> region(gm);
    soapgb_maps maps{delta.data(), limb.data(), mu.data(), region.data(), lb.data()};
    tool::check(ctx, soapgb_disk_maps(ctx, &st, n_mu, mu_b.data(), SOAPGB_HOST, &maps), "disk maps");

    std::vector<double> quiet(n, 0.0);
    tool::check(ctx,
                soapgb_quiet_disk(ctx, form, n, (int)n_eff, wave.data(), cube.data(), n_mu, st.grid, delta.data(),
                                  limb.data(), region.data(), step, SOAPGB_HOST, quiet.data()),
                "quiet disk");

    // lower_resolution_gpu(..., wavelength_step_median, window_width, ...): the
    // exponent keeps the reference's literal 0.005 (SOAP_initialize.cu:87)
    std::vector<double> low(n_eff);
    tool::check(ctx,
                soapgb_lower_resolution(ctx, form, n, (int)n_eff, 1, wave.data(), nullptr, quiet.data(), sigma_v,
                                        window, step_median, 0.005, -60000.0, SOAPGB_HOST, low.data(), nullptr),
                "lower resolution");

    tool::write_bin(prefix + "mu_map.bin", mu.data(), gm);
    tool::write_bin(prefix + "delta_map.bin", delta.data(), gm);
    tool::write_bin(prefix + "limb_map.bin", limb.data(), gm);
    tool::write_bin(prefix + "region_map.bin", region.data(), gm);
    tool::write_bin(prefix + "LB_map.bin", lb.data(), gm);
    tool::write_bin(prefix + "_quiet_sun_lower_spec.bin", low.data(), n_eff);
    tool::write_bin(prefix + "_quiet_sun_spec.bin", quiet.data(), n_eff);
    tool::write_bin(prefix + "_quiet_sun_wave.bin", wave.data(), n_eff);
    soapgb_ctx_destroy(ctx);
    timer.report();
    return 0;
}
