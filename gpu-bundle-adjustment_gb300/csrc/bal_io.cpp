// BAL text reader / writer and the CPU Snavely residual of the drop-in API.
//
// Format and validation follow the reference reader (src/bal_reader.cpp:12-98):
// header "C P E", E lines "camera point x y", 9C camera values, 3P point
// values; whitespace-separated; .bz2 input is decompressed by `bzcat`; a bad
// header, an out-of-range index, a malformed number or trailing data throws.
// The residual follows src/bal_reader.cpp:100-128 (rotation applied when
// |rodrigues| > 1e-12, else P = X + t).

#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>

#include "gba/bal_problem.hpp"

namespace gba {
namespace {

bool ends_with(const std::string& s, const char* suf) {
    const size_t n = std::strlen(suf);
    return s.size() >= n && s.compare(s.size() - n, n, suf) == 0;
}

std::string slurp(const std::string& path) {
    const bool bz = ends_with(path, ".bz2");
    FILE* fp = nullptr;
    if (bz) {
        if (path.find('"') != std::string::npos || path.find('`') != std::string::npos ||
            path.find('$') != std::string::npos)
            throw std::runtime_error("unsupported characters in path " + path);
        const std::string cmd = "bzcat -- \"" + path + "\"";
        fp = popen(cmd.c_str(), "r");
    } else {
        fp = std::fopen(path.c_str(), "rb");
    }
    if (!fp) throw std::runtime_error("cannot open " + path);
    std::string text;
    std::string chunk(1 << 20, '\0');
    size_t got;
    while ((got = std::fread(&chunk[0], 1, chunk.size(), fp)) > 0) text.append(chunk.data(), got);
    const int rc = bz ? pclose(fp) : std::fclose(fp);
    if (rc != 0) throw std::runtime_error("read failed for " + path);
    return text;
}

class Tokens {
public:
    explicit Tokens(const std::string& t) : p_(t.data()), end_(t.data() + t.size()) {}
    template <typename T>
    T get() {
        skip();
        T v{};
        const auto res = std::from_chars(p_, end_, v);
        if (res.ec != std::errc()) throw std::runtime_error("malformed BAL number");
        p_ = res.ptr;
        return v;
    }
    bool done() {
        skip();
        return p_ == end_;
    }

private:
    void skip() {
        while (p_ != end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) ++p_;
    }
    const char* p_;
    const char* end_;
};

}  // namespace

BALProblem load_bal(const std::string& path) {
    const std::string text = slurp(path);
    Tokens tok(text);
    BALProblem p;
    p.num_cameras = tok.get<int>();
    p.num_points = tok.get<int>();
    p.num_observations = tok.get<int>();
    if (p.num_cameras <= 0 || p.num_points <= 0 || p.num_observations <= 0)
        throw std::runtime_error("bad BAL header in " + path);
    const size_t E = static_cast<size_t>(p.num_observations);
    p.obs_camera.resize(E);
    p.obs_point.resize(E);
    p.obs_pixel.resize(2 * E);
    for (size_t i = 0; i < E; ++i) {
        const int c = tok.get<int>();
        const int q = tok.get<int>();
        if (c < 0 || c >= p.num_cameras || q < 0 || q >= p.num_points)
            throw std::runtime_error("observation index out of range in " + path);
        p.obs_camera[i] = c;
        p.obs_point[i] = q;
        p.obs_pixel[2 * i] = tok.get<double>();
        p.obs_pixel[2 * i + 1] = tok.get<double>();
    }
    p.cameras.resize(9 * static_cast<size_t>(p.num_cameras));
    for (double& v : p.cameras) v = tok.get<double>();
    p.points.resize(3 * static_cast<size_t>(p.num_points));
    for (double& v : p.points) v = tok.get<double>();
    if (!tok.done()) throw std::runtime_error("trailing garbage in " + path);
    return p;
}

void write_bal(const std::string& path, const BALProblem& p) {
    FILE* fp = std::fopen(path.c_str(), "w");
    if (!fp) throw std::runtime_error("cannot write " + path);
    std::fprintf(fp, "%d %d %d\n", p.num_cameras, p.num_points, p.num_observations);
    for (int i = 0; i < p.num_observations; ++i)
        std::fprintf(fp, "%d %d %.17g %.17g\n", p.obs_camera[i], p.obs_point[i], p.obs_pixel[2 * i],
                     p.obs_pixel[2 * i + 1]);
    for (double v : p.cameras) std::fprintf(fp, "%.17g\n", v);
    for (double v : p.points) std::fprintf(fp, "%.17g\n", v);
    if (std::fclose(fp) != 0) throw std::runtime_error("write failed for " + path);
}

void snavely_residual(const double* camera9, const double* point3, const double* observed2, double* out2) {
    const double* a = camera9;
    const double* X = point3;
    const double th = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    double P[3];
    if (th > 1e-12) {
        const double w0 = a[0] / th, w1 = a[1] / th, w2 = a[2] / th;
        const double c = std::cos(th), s = std::sin(th);
        const double wX = w0 * X[0] + w1 * X[1] + w2 * X[2];
        const double k = wX * (1.0 - c);
        P[0] = X[0] * c + (w1 * X[2] - w2 * X[1]) * s + w0 * k + camera9[3];
        P[1] = X[1] * c + (w2 * X[0] - w0 * X[2]) * s + w1 * k + camera9[4];
        P[2] = X[2] * c + (w0 * X[1] - w1 * X[0]) * s + w2 * k + camera9[5];
    } else {
        P[0] = X[0] + camera9[3];
        P[1] = X[1] + camera9[4];
        P[2] = X[2] + camera9[5];
    }
    const double u = -P[0] / P[2], v = -P[1] / P[2];
    const double r2 = u * u + v * v;
    const double d = 1.0 + camera9[7] * r2 + camera9[8] * r2 * r2;
    out2[0] = camera9[6] * d * u - observed2[0];
    out2[1] = camera9[6] * d * v - observed2[1];
}

double total_squared_error(const BALProblem& p) {
    double sum = 0.0;
    double r[2];
    for (int i = 0; i < p.num_observations; ++i) {
        snavely_residual(p.camera(p.obs_camera[i]), p.point(p.obs_point[i]), &p.obs_pixel[2 * static_cast<size_t>(i)], r);
        sum += r[0] * r[0] + r[1] * r[1];
    }
    return sum;
}

}  // namespace gba
