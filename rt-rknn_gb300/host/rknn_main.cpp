// rknn-gb300: command-line drop-in for the reference's query binaries.
//
//   rknn-gb300 -if <file> -k <k> -q <index> [-al <name>] [--mode fp64|fp32]
//              [--queries i,j,...] [--log <dir>] [--no-log] [--save <snapshot>]
//
// The input file may also be a binary index snapshot (rknn_snapshot_write's
// format, recognised by its magic), which loads without parsing; --save
// writes one of the loaded points.
// Same options and defaults as rknn-inf (rknn-inf/inf.cpp:38-119: -if/--infile,
// -k (default 4), -q (default 0, an index into the facility list), -al parsed
// and ignored), same input format (inf.cpp:129-161), and the reference's
// summary lines on stdout.  In addition it writes the result set of each
// query to <log>/<mode>_k<k>_q<q>.txt, one user id per line in ascending
// order (the reference's README promises result files in log/ but its
// binaries only print counts).  Exit status 1 on any error.
#include "rknn_gpu.h"

#include <sys/stat.h>
#include <sys/time.h>

#include <charconv>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

double wall()
{
    timeval t;
    gettimeofday(&t, nullptr);
    return (double)t.tv_sec + (double)t.tv_usec * 1e-6;
}

[[noreturn]] void usage(const char* argv0)
{
    std::fprintf(stderr,
                 "Usage  : %s [options]\n"
                 "Options: --infile | -if <filename>   input file (facilities then users)\n"
                 "         -k <k>                      k (default 4)\n"
                 "         -q <index>                  query facility index (default 0)\n"
                 "         --algorithm | -al <name>    accepted and ignored\n"
                 "         --mode fp64|fp32            predicate filter precision (default fp64)\n"
                 "         --filter inf|slice|auto     candidate filter (default inf: rknn-inf's\n"
                 "                                     influence zone; slice: angular slices)\n"
                 "         --queries i,j,...           several query indices in one batch\n"
                 "         --log <dir>                 result directory (default log)\n"
                 "         --no-log                    do not write result files\n"
                 "         --save <file>               also write the points as a binary snapshot\n"
                 "                                     (a later -if loads it without parsing)\n"
                 "         --help | -h                 print this message\n",
                 argv0);
    std::exit(1);
}

struct Parser {
    const char* p;
    const char* end;
    // the next whitespace-separated token as [b, e)
    bool span(const char*& b, const char*& e)
    {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r')) ++p;
        if (p >= end) return false;
        b = p;
        while (p < end && !(*p == ' ' || *p == '\n' || *p == '\t' || *p == '\r')) ++p;
        e = p;
        return true;
    }
    bool next(std::string& tok)
    {
        const char *b, *e;
        if (!span(b, e)) return false;
        tok.assign(b, e - b);
        return true;
    }
};

// A token as an integer / a double: std::from_chars on the buffer (no
// copies, no locale), strtoll / strtod for the forms it does not take (a
// leading '+', hexadecimal floats, inf / nan); both give the correctly
// rounded double, as the reference's stream extraction does.
bool parse_int(const char* b, const char* e, long long& v)
{
    const auto r = std::from_chars(b, e, v);
    if (r.ec == std::errc() && r.ptr == e) return true;
    std::string t(b, e);
    char* x;
    errno = 0;
    v = std::strtoll(t.c_str(), &x, 10);
    return !*x && !errno && !t.empty();
}

bool parse_double(const char* b, const char* e, double& v)
{
    const auto r = std::from_chars(b, e, v);
    if (r.ec == std::errc() && r.ptr == e) return true;
    std::string t(b, e);
    char* x;
    v = std::strtod(t.c_str(), &x);
    return !*x && !t.empty();
}

bool read_file(const std::string& path, std::string& data)
{
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    data.resize(n > 0 ? (size_t)n : 0);
    size_t got = n > 0 ? std::fread(&data[0], 1, (size_t)n, f) : 0;
    std::fclose(f);
    return got == data.size();
}

bool parse_points(Parser& ps, long long n, std::vector<float>& xy, std::vector<int32_t>& id,
                  long long& inexact)
{
    xy.resize(2 * n);
    id.resize(n);
    const char *b, *e;
    for (long long i = 0; i < n; ++i) {
        long long v;
        if (!ps.span(b, e) || !parse_int(b, e, v)) return false;
        id[i] = (int32_t)v;
        for (int c = 0; c < 2; ++c) {
            double d;
            if (!ps.span(b, e) || !parse_double(b, e, d)) return false;
            float f = (float)d;
            if ((double)f != d) ++inexact;
            xy[2 * i + c] = f;
        }
    }
    return true;
}

}  // namespace

int main(int argc, char** argv)
{
    std::string infile, logdir = "log", mode_s = "fp64", filter_s = "inf", save_path;
    long long k = 4, q = 0;
    std::vector<long long> queries;
    bool write_log = true;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto val = [&]() -> std::string {
            if (i + 1 >= argc) usage(argv[0]);
            return argv[++i];
        };
        if (a == "--help" || a == "-h") usage(argv[0]);
        else if (a == "--infile" || a == "-if") infile = val();
        else if (a == "--algorithm" || a == "-al") (void)val();
        else if (a == "-k") {
            k = std::atoll(val().c_str());
            if (k <= 0) {
                std::fprintf(stderr, "Invalid value for k: %lld. It must be a positive integer.\n", k);
                return 1;
            }
        } else if (a == "-q") {
            q = std::atoll(val().c_str());
            if (q < 0) {
                std::fprintf(stderr, "Invalid value for q: %lld. It must be a >= 0 number.\n", q);
                return 1;
            }
        } else if (a == "--mode") mode_s = val();
        else if (a == "--filter") filter_s = val();
        else if (a == "--queries") {
            std::string s = val();
            size_t b = 0;
            while (b <= s.size()) {
                size_t e = s.find(',', b);
                if (e == std::string::npos) e = s.size();
                if (e > b) queries.push_back(std::atoll(s.substr(b, e - b).c_str()));
                b = e + 1;
            }
        } else if (a == "--log") logdir = val();
        else if (a == "--no-log") write_log = false;
        else if (a == "--save") save_path = val();
        else {
            std::fprintf(stderr, "Unknown option '%s'\n", a.c_str());
            usage(argv[0]);
        }
    }
    if (mode_s != "fp64" && mode_s != "fp32") {
        std::fprintf(stderr, "Unknown mode '%s'\n", mode_s.c_str());
        return 1;
    }
    const int mode = mode_s == "fp32" ? RKNN_MODE_FP32 : RKNN_MODE_FP64;
    if (filter_s != "inf" && filter_s != "slice" && filter_s != "auto") {
        std::fprintf(stderr, "Unknown filter '%s'\n", filter_s.c_str());
        return 1;
    }
    rknn_index_opts opts;
    rknn_index_opts_default(&opts);
    opts.filter = filter_s == "inf" ? RKNN_FILTER_INF : filter_s == "slice" ? RKNN_FILTER_SLICE : RKNN_FILTER_AUTO;
    if (queries.empty()) queries.push_back(q);

    std::printf("Loading data...\n");
    std::string data;
    if (!read_file(infile, data)) {
        std::fprintf(stderr, "Error opening file: %s\n", infile.c_str());
        return 1;
    }
    std::vector<float> fxy, uxy;
    std::vector<int32_t> fid, uid;
    long long inexact = 0, nf = 0, nu = 0;
    if (data.size() >= 8 && std::memcmp(data.data(), "RKNNSNP1", 8) == 0) {
        // a binary snapshot: read by the library (checked against its hash)
        data.clear();
        data.shrink_to_fit();
        float *a = nullptr, *c = nullptr;
        int32_t *b = nullptr, *d = nullptr;
        int64_t n1 = 0, n2 = 0;
        if (rknn_snapshot_read(infile.c_str(), &a, &b, &n1, &c, &d, &n2) != RKNN_OK) {
            std::fprintf(stderr, "Error reading snapshot: %s\n", rknn_last_error());
            return 1;
        }
        nf = n1;
        nu = n2;
        fxy.assign(a, a + 2 * n1); fid.assign(b, b + n1);
        uxy.assign(c, c + 2 * n2); uid.assign(d, d + n2);
        rknn_snapshot_free(a); rknn_snapshot_free(b); rknn_snapshot_free(c); rknn_snapshot_free(d);
    } else {
        Parser ps{data.data(), data.data() + data.size()};
        std::string t;
        if (!ps.next(t) || (nf = std::atoll(t.c_str())) < 1 || !parse_points(ps, nf, fxy, fid, inexact) ||
            !ps.next(t) || (nu = std::atoll(t.c_str())) < 0 || !parse_points(ps, nu, uxy, uid, inexact)) {
            std::fprintf(stderr, "Error parsing file: %s\n", infile.c_str());
            return 1;
        }
    }
    if (!save_path.empty() &&
        rknn_snapshot_write(save_path.c_str(), fxy.data(), fid.data(), nf, uxy.data(), uid.data(), nu) != RKNN_OK) {
        std::fprintf(stderr, "Error writing snapshot: %s\n", rknn_last_error());
        return 1;
    }
    std::printf("Loaded %lld facilities and %lld users.\n", nf, nu);
    if (inexact)
        std::fprintf(stderr, "warning: %lld coordinates are not float32 values and were rounded\n", inexact);
    for (long long qq : queries)
        if (qq < 0 || qq >= nf) {
            std::fprintf(stderr, "Invalid value for q: %lld (there are %lld facilities)\n", qq, nf);
            return 1;
        }

    std::printf("building grid index...\n");
    double t0 = wall();
    rknn_index* ix = nullptr;
    if (rknn_index_create(fxy.data(), fid.data(), nf, uxy.data(), uid.data(), nu, &opts, &ix) != RKNN_OK) {
        std::fprintf(stderr, "index build failed: %s\n", rknn_last_error());
        return 1;
    }
    std::printf("Grid index is built in %g[s].\n\n", wall() - t0);

    std::vector<int32_t> qv(queries.begin(), queries.end()), kv(queries.size(), (int32_t)k);
    std::vector<int64_t> off(queries.size() + 1);
    std::vector<int32_t> ids((size_t)nu + 1);
    rknn_query_stats st;
    t0 = wall();
    rknn_status s = rknn_query_batch(ix, qv.data(), kv.data(), (int32_t)qv.size(), mode, ids.data(),
                                     (int64_t)ids.size(), off.data(), &st);
    if (s == RKNN_ERR_CAPACITY) {
        ids.resize((size_t)off.back());
        s = rknn_query_batch(ix, qv.data(), kv.data(), (int32_t)qv.size(), mode, ids.data(),
                             (int64_t)ids.size(), off.data(), &st);
    }
    double elapsed = wall() - t0;
    if (s != RKNN_OK) {
        std::fprintf(stderr, "query failed: %s\n", rknn_last_error());
        rknn_index_destroy(ix);
        return 1;
    }
    if (write_log) {
        mkdir(logdir.c_str(), 0755);
    }
    for (size_t i = 0; i < qv.size(); ++i) {
        int32_t nb = 0, fl = 0;
        rknn_last_zone(ix, (int32_t)i, nullptr, 0, &nb, &fl);
        long long n = off[i + 1] - off[i];
        if (qv.size() > 1) std::printf("Query %d:\n", qv[i]);
        std::printf("Total bisectors created: %d\n", nb);
        std::printf("Found %lld RkNN results.\n", n);
        if (write_log) {
            std::string path = logdir + "/" + mode_s + "_k" + std::to_string(k) + "_q" + std::to_string(qv[i]) + ".txt";
            FILE* f = std::fopen(path.c_str(), "w");
            if (!f) {
                std::fprintf(stderr, "cannot write %s\n", path.c_str());
                rknn_index_destroy(ix);
                return 1;
            }
            for (long long j = off[i]; j < off[i + 1]; ++j) std::fprintf(f, "%d\n", ids[j]);
            std::fclose(f);
        }
    }
    std::printf("Device time: %g[s].\n", st.device_ms * 1e-3);
    std::printf("Total time: %g[s].\n\n", elapsed);
    rknn_index_destroy(ix);
    return 0;
}
