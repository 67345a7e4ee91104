// Drop-in SOAP_integration (and, built with -DSOAPGB_SOLAR=1, SOAP_integration_solar):
// the argv / file contract of SOAP_integration.cu:464-860 on top of libsoapgb
// (soapgb_phase_maps, soapgb_phase_integrate).
//
// argv: G nrho n_phase T_star dT_spot I dT_fac phase_locator.txt fac_cube.bin N raw_dir
//       maps_dir no_block no_thread quiet_cube.bin spot_cube.bin file_prefix step n_mu
//       wave.bin quiet_SED.bin spot_conti.bin fac_conti.bin map_dir/
// reads:  maps_dir/final_info.txt, maps_dir/maps<id>_for_all.txt,
//         map_dir/<prefix>{region,delta,limb,LB}_map.bin
// writes: raw_dir/<prefix>_Spec_{flux,bconv,tot}_<id>_.bin,
//         raw_dir/<prefix>_{temp_map,spot_binary_map}_<id>_.bin
#include <algorithm>

#include "tool_common.h"

#ifndef SOAPGB_SOLAR
#define SOAPGB_SOLAR 0
#endif

int main(int argc, char *argv[]) {
    tool::Timer timer;
    tool::need_args(argc, 24,
                    "G nrho n_phase T_star dT_spot I dT_fac phase_locator.txt fac_cube.bin N raw_dir maps_dir "
                    "no_block no_thread quiet_cube.bin spot_cube.bin file_prefix step n_mu wave.bin quiet_SED.bin "
                    "spot_conti.bin fac_conti.bin map_dir/");
    int grid = std::atoi(argv[1]);
    soapgb_activity act;
    act.nrho = std::atoi(argv[2]);
    int npsi = std::atoi(argv[3]);
    act.t_star = std::atoi(argv[4]);
    act.t_diff_spot = std::atoi(argv[5]);
    double incl = std::atof(argv[6]);
    act.t_diff_fac = std::atoi(argv[7]);
    act.solar = SOAPGB_SOLAR;
    std::string phase_name = argv[8];
    std::string fac_name = argv[9];
    int n = std::atoi(argv[10]);
    std::string out_dir = argv[11];
    std::string map_dir = argv[12];
    int no_block = std::atoi(argv[13]);
    int no_thread = std::atoi(argv[14]);
    std::string quiet_name = argv[15];
    std::string spot_name = argv[16];
    std::string prefix = argv[17];
    double step = std::atof(argv[18]);
    int n_mu = std::atoi(argv[19]);
    std::string wave_name = argv[20];
    std::string qsed_name = argv[21];
    std::string spot_sed_name = argv[22];
    std::string fac_sed_name = argv[23];
    std::string map_soap_dir = argv[24];
    long long n_eff = (long long)no_block * no_thread;
    if (grid < 1 || npsi < 0 || n < 3 || n_mu < 1 || n_eff < 2 || n_eff > n)
        tool::die("inconsistent sizes: N=" + std::to_string(n) + " no_block*no_thread=" + std::to_string(n_eff));
    int form = tool::form_from_env();
    size_t cn = (size_t)n * n_mu;
    std::vector<double> q_sed = tool::read_f64(qsed_name, cn);
    std::vector<double> spot_sed = tool::read_f64(spot_sed_name, cn);
    std::vector<double> fac_sed = tool::read_f64(fac_sed_name, cn);
    std::vector<double> q_norm = tool::read_f64(quiet_name, cn);
    std::vector<double> wave = tool::read_f64(wave_name, n);
    std::vector<double> spot_norm = tool::read_f64(spot_name, cn);
    std::vector<double> fac_norm = tool::read_f64(fac_name, cn);
    long long gm = (long long)grid * grid;
    std::string mp = map_soap_dir + prefix;
    std::vector<int> region = tool::read_i32(mp + "region_map.bin", gm);
    std::vector<double> delta = tool::read_f64(mp + "delta_map.bin", gm);
    std::vector<double> limb = tool::read_f64(mp + "limb_map.bin", gm);
    std::vector<double> lbv = tool::read_f64(mp + "LB_map.bin", gm);
    std::vector<double> psi = tool::read_text(phase_name, npsi);
    std::vector<double> info = tool::read_text(map_dir + "final_info.txt", 2 * (size_t)npsi);
    // region tables, SOAP_integration.cu:661-682
    std::vector<int> ids(npsi), off(npsi + 1, 0);
    std::vector<double> regions;
    for (int p = 0; p < npsi; ++p) {
        ids[p] = (int)info[2 * p];
        int m = (int)info[2 * p + 1];
        std::vector<double> rows =
            m > 0 ? tool::read_text(map_dir + "maps" + std::to_string(ids[p]) + "_for_all.txt", 4 * (size_t)m)
                  : std::vector<double>();
        regions.insert(regions.end(), rows.begin(), rows.end());
        off[p + 1] = off[p] + m;
    }
    soapgb_ctx *ctx = tool::open_ctx();
    soapgb_maps maps{delta.data(), limb.data(), nullptr, region.data(), lbv.data()};
    soapgb_cubes cubes{q_norm.data(), q_sed.data(), spot_norm.data(), fac_norm.data(), spot_sed.data(),
                       fac_sed.data(), n_mu};
    // phases in chunks to bound host memory
    const int chunk = 32;
    for (int p0 = 0; p0 < npsi; p0 += chunk) {
        int np = std::min(chunk, npsi - p0);
        std::vector<int> coff(np + 1);
        for (int q = 0; q <= np; ++q) coff[q] = off[p0 + q] - off[p0];
        std::vector<double> temp(gm * np), bi(gm * np);
        const double *rg = regions.empty() ? nullptr : regions.data() + 4 * (size_t)off[p0];
        tool::check(ctx,
                    soapgb_phase_maps(ctx, grid, incl, np, psi.data() + p0, coff.data(), rg, &act, SOAPGB_HOST,
                                      temp.data(), bi.data()),
                    "phase maps");
        std::vector<double> flux((size_t)n * np), bconv((size_t)n * np), tot((size_t)n * np);
        tool::check(ctx,
                    soapgb_phase_integrate(ctx, form, n, (int)n_eff, wave.data(), grid, np, temp.data(), bi.data(),
                                           &maps, &cubes, step, &act, SOAPGB_HOST, flux.data(), bconv.data(),
                                           tot.data()),
                    "phase integration");
        for (int q = 0; q < np; ++q) {
            std::string id = std::to_string(ids[p0 + q]);
            size_t o = (size_t)n * q;
            tool::write_bin(out_dir + prefix + "_Spec_flux_" + id + "_.bin", flux.data() + o, n_eff);
            tool::write_bin(out_dir + prefix + "_Spec_bconv_" + id + "_.bin", bconv.data() + o, n_eff);
            std::string tot_name = out_dir + prefix + "_Spec_tot_" + id + "_.bin";
            tool::write_bin(tot_name, tot.data() + o, n_eff);
            std::cout << tot_name << std::endl;
            tool::write_bin(out_dir + prefix + "_temp_map_" + id + "_.bin", temp.data() + gm * q, gm);
            tool::write_bin(out_dir + prefix + "_spot_binary_map_" + id + "_.bin", bi.data() + gm * q, gm);
        }
    }
    soapgb_ctx_destroy(ctx);
    timer.report();
    return 0;
}
