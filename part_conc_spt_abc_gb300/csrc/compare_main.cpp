/*
 * compare -- population averages of two output.xml files side by side.
 *
 *     compare a.xml b.xml
 *
 * The reference ships this tool (src/compare_output/compare.cpp) but its
 * output::load is a stub, so it cannot run there; here it reads the files
 * with pcs_output_load.  It prints, for m, c, az, dist and w, the mean over
 * all entries of each file and the absolute difference, then the two
 * epsilons, one line each in the reference tool's format; with a wrong
 * argument count it prints the reference's error and returns 1, and a file
 * that does not load prints "Top-level exception: <type>" and the message.
 */
#include <cmath>
#include <cstdio>
#include <string>

#include "../../include/pcs.h"

namespace {

double mean_of(const double* x, size_t n)
{
    double acc = 0.0, cnt = 0.0;
    for (size_t i = 0; i < n; ++i, cnt += 1.0) acc += x[i];
    return acc / cnt;
}

void line(const char* name, double a, double b)
{
    std::printf("%s: %18g vs %18g (\xce\xb4 = %18g)\n", name, a, b, std::fabs(a - b));
}

int load(const char* path, pcs_output** o)
{
    const pcs_status s = pcs_output_load(path, o);
    if (s == PCS_OK) return 0;
    const char* type = s == PCS_ERR_XML ? "error::XMLLoadError" : "error::RuntimeError";
    std::fprintf(stderr, "Top-level exception: %s\n", type);
    std::fprintf(stderr, "  - %s: %s\n", pcs_status_string(s), pcs_last_error());
    return 1;
}

} // namespace

int main(int argc, char** argv)
{
    if (argc != 3) {
        std::fprintf(stderr, "Error: need exactly two command line args.\n");
        return 1;
    }
    pcs_output *a = nullptr, *b = nullptr;
    if (load(argv[1], &a)) return 1;
    if (load(argv[2], &b)) {
        pcs_output_free(a);
        return 1;
    }
    pcs_output_view va, vb;
    pcs_output_get(a, &va);
    pcs_output_get(b, &vb);
    line("m    ", mean_of(va.m, va.nm), mean_of(vb.m, vb.nm));
    line("c    ", mean_of(va.c, va.nc), mean_of(vb.c, vb.nc));
    line("az   ", mean_of(va.az, va.naz), mean_of(vb.az, vb.naz));
    line("dist ", mean_of(va.dist, va.nd), mean_of(vb.dist, vb.nd));
    line("w    ", mean_of(va.w, va.nw), mean_of(vb.w, vb.nw));
    line("eps  ", va.gamma, vb.gamma);
    pcs_output_free(a);
    pcs_output_free(b);
    return 0;
}
