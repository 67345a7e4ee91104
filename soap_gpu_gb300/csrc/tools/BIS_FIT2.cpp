// Drop-in BIS_FIT2: the argv / file contract of BIS_FIT2.cpp:97-320 on top of
// libsoapgb (soapgb_gauss_bis with one spectrum).  The batched form of the same
// call is what the in-process driver uses for all spectra at once.
//
// argv: n
// reads:  CCF_data.txt (n rows: velocity, ccf), CCF_error.txt (n values)
// writes: ccf_model.bin (n), ccf_parameter.bin (c, |k|, span, v0, fwhm),
//         ccf_depth.bin (91), ccf_bis.bin (91)
#include "tool_common.h"

int main(int argc, char *argv[]) {
    tool::need_args(argc, 1, "n");
    int n = std::atoi(argv[1]);
    if (n < 8) tool::die("need at least 8 CCF points");
    std::vector<double> xy = tool::read_text("CCF_data.txt", 2 * (size_t)n);
    std::vector<double> err = tool::read_text("CCF_error.txt", n);
    std::vector<double> x(n), y(n);
    for (int i = 0; i < n; ++i) {
        x[i] = xy[2 * i];
        y[i] = xy[2 * i + 1];
    }
    soapgb_ctx *ctx = tool::open_ctx();
    std::vector<double> model(n), par(5), depth(91), bis(91);
    int iters = 0;
    tool::check(ctx,
                soapgb_gauss_bis(ctx, 1, n, x.data(), y.data(), err.data(), SOAPGB_HOST, model.data(), par.data(),
                                 depth.data(), bis.data(), &iters),
                "gauss fit");
    soapgb_ctx_destroy(ctx);
    tool::write_bin("ccf_model.bin", model.data(), n);
    tool::write_bin("ccf_parameter.bin", par.data(), 5);
    tool::write_bin("ccf_depth.bin", depth.data(), 91);
    tool::write_bin("ccf_bis.bin", bis.data(), 91);
    return 0;
}
