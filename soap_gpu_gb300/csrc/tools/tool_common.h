// Shared helpers of the argv-compatible executables (file I/O, context, errors).
#pragma once

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "soapgb.h"

namespace tool {

[[noreturn]] inline void die(const std::string &msg) {
    std::fprintf(stderr, "error: %s\n", msg.c_str());
    std::exit(1);
}

inline void need_args(int argc, int want, const char *usage) {
    if (argc < want + 1) die(std::string("expected ") + std::to_string(want) + " arguments: " + usage);
}

// Reads `count` float64 values; fails loudly on a missing or short file (the
// reference's fread silently leaves garbage in that case).
inline std::vector<double> read_f64(const std::string &path, size_t count, size_t pad_to = 0) {
    std::vector<double> v(pad_to > count ? pad_to : count, 0.0);
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) die("cannot open " + path);
    size_t got = std::fread(v.data(), sizeof(double), count, f);
    std::fclose(f);
    if (got != count) die(path + ": expected " + std::to_string(count) + " float64 values, found " + std::to_string(got));
    return v;
}

inline std::vector<int> read_i32(const std::string &path, size_t count) {
    std::vector<int> v(count, 0);
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) die("cannot open " + path);
    size_t got = std::fread(v.data(), sizeof(int), count, f);
    std::fclose(f);
    if (got != count) die(path + ": expected " + std::to_string(count) + " int32 values, found " + std::to_string(got));
    return v;
}

template <class T>
inline void write_bin(const std::string &path, const T *p, size_t count) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) die("cannot create " + path);
    size_t put = std::fwrite(p, sizeof(T), count, f);
    std::fclose(f);
    if (put != count) die("short write to " + path);
}

// whitespace-separated numbers
inline std::vector<double> read_text(const std::string &path, size_t count) {
    std::ifstream in(path);
    if (!in) die("cannot open " + path);
    std::vector<double> v(count);
    for (size_t i = 0; i < count; ++i)
        if (!(in >> v[i])) die(path + ": expected " + std::to_string(count) + " numbers");
    return v;
}

inline void check(soapgb_ctx *ctx, int rc, const char *what) {
    if (rc != SOAPGB_OK) die(std::string(what) + ": " + soapgb_last_error(ctx));
}

inline soapgb_ctx *open_ctx() {
    soapgb_ctx *ctx = nullptr;
    int dev = 0;
    if (const char *e = std::getenv("SOAPGB_DEVICE")) dev = std::atoi(e);
    int rc = soapgb_ctx_create(dev, &ctx);
    if (rc != SOAPGB_OK) die(std::string("no usable CUDA device: ") + (ctx ? soapgb_last_error(ctx) : "?"));
    return ctx;
}

// arithmetic form: SOAPGB_FORM = plain64 (default, the reference's arithmetic),
// fast64 or fast32
inline int form_from_env() {
    const char *e = std::getenv("SOAPGB_FORM");
    if (!e || !*e || !std::strcmp(e, "plain64")) return SOAPGB_PLAIN64;
    if (!std::strcmp(e, "fast64")) return SOAPGB_FAST64;
    if (!std::strcmp(e, "fast32")) return SOAPGB_FAST32;
    die(std::string("SOAPGB_FORM must be plain64, fast64 or fast32 (got ") + e + ")");
}

struct Timer {
    std::chrono::system_clock::time_point wall = std::chrono::system_clock::now();
    std::clock_t cpu = std::clock();
    void report() const {
        std::chrono::duration<double> d = std::chrono::system_clock::now() - wall;
        std::cout << "finished in " << d.count() << " seconds [wall clock]" << std::endl;
        std::cout << "time: " << double(std::clock() - cpu) / double(CLOCKS_PER_SEC) << std::endl;
    }
};

}  // namespace tool
