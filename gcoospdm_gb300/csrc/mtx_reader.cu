// mtx_reader.cu -- Matrix Market input on the host: the reference driver's
// -file= reader (src/MatrixReader.cpp:11-84) as COO triplets for
// gcoo_create_coo, without the dense m x k buffer the reference fills.
// Host code only (no kernels).
//
// Semantics kept: 1-based indices, entries in file order, every non-general
// matrix mirrored (the mirror of an entry right after it), so a later
// duplicate wins in gcoo_create_coo as it does in the reference's dense
// buffer, and explicit zeros are dropped by the build's `v != 0` test.
// Differences, both where the reference's values are not the matrix's:
// pattern entries are 1.0 (the reference draws unseeded rand() values), and
// the mirror of a skew-symmetric entry is negated, as the format defines.
// "hermitian" is read like "symmetric": for the real, integer and pattern
// fields read here the conjugate of a value is the value itself (the
// reference mirrors every banner that does not say "general").
//
// No C++ exception leaves the entry point: a host allocation that fails
// while the triplets grow returns GCOO_ERROR_ALLOC, anything else thrown
// GCOO_ERROR_INVALID_VALUE.
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <cctype>
#include <new>
#include <string>
#include <vector>

#include "internal.cuh"

namespace gcoo {
namespace {

std::string lower(std::string s)
{
    std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return static_cast<char>(std::tolower(c)); });
    return s;
}

bool blank(const char *p)
{
    while (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\n')
        ++p;
    return *p == 0;
}

// A line of any length (getline grows the buffer); false at the end of file.
bool next_line(FILE *f, char **buf, size_t *cap) { return getline(buf, cap, f) >= 0; }

struct FileCloser {
    FILE *f;
    char *line = nullptr;
    ~FileCloser()
    {
        free(line);
        if (f)
            fclose(f);
    }
};

// The reader proper; its std::vector / std::string work may throw.
gcoo_status read_matrix_market(const char *path, int64_t *m, int64_t *k, int64_t *count, int32_t **rows,
                               int32_t **cols, float **vals)
{
    FileCloser fc{fopen(path, "r")};
    if (!fc.f)
        return fail(GCOO_ERROR_INVALID_VALUE, std::string("cannot open ") + path + ": " + strerror(errno));
    size_t cap = 0;
    if (!next_line(fc.f, &fc.line, &cap))
        return fail(GCOO_ERROR_INVALID_VALUE, "empty file");
    // banner: %%MatrixMarket matrix <format> <field> <symmetry>
    char w[5][64] = {};
    if (sscanf(fc.line, "%63s %63s %63s %63s %63s", w[0], w[1], w[2], w[3], w[4]) != 5 ||
        lower(w[0]) != "%%matrixmarket" || lower(w[1]) != "matrix")
        return fail(GCOO_ERROR_INVALID_VALUE, "not a Matrix Market matrix banner");
    const std::string format = lower(w[2]), field = lower(w[3]), symmetry = lower(w[4]);
    if (format != "coordinate")
        return fail(GCOO_ERROR_UNSUPPORTED, "only the coordinate format is read (got " + format + ")");
    if (field != "real" && field != "integer" && field != "pattern" && field != "double")
        return fail(GCOO_ERROR_UNSUPPORTED, "field " + field + " is not read (real, integer or pattern)");
    int mirror = 0; // 0 general, 1 symmetric, -1 skew-symmetric
    if (symmetry == "symmetric")
        mirror = 1;
    else if (symmetry == "hermitian") // real-valued fields: the same as symmetric
        mirror = 1;
    else if (symmetry == "skew-symmetric")
        mirror = -1;
    else if (symmetry != "general")
        return fail(GCOO_ERROR_UNSUPPORTED, "symmetry " + symmetry + " is not read");
    const bool pattern = field == "pattern";

    // comments, then the size line
    bool have_size = false;
    long long nr = 0, nc = 0, ne = 0;
    while (next_line(fc.f, &fc.line, &cap)) {
        if (fc.line[0] == '%' || blank(fc.line))
            continue;
        if (sscanf(fc.line, "%lld %lld %lld", &nr, &nc, &ne) != 3)
            return fail(GCOO_ERROR_INVALID_VALUE, "malformed size line");
        have_size = true;
        break;
    }
    if (!have_size)
        return fail(GCOO_ERROR_INVALID_VALUE, "no size line");
    if (nr <= 0 || nc <= 0 || ne < 0)
        return fail(GCOO_ERROR_INVALID_VALUE, "sizes must be positive and the entry count non-negative");
    if (nr > 0x7fffffffLL || nc > 0x7fffffffLL)
        return fail(GCOO_ERROR_FORMAT, "dimensions beyond int32");
    if (mirror != 0 && nr != nc)
        return fail(GCOO_ERROR_INVALID_VALUE, "a symmetric matrix must be square");

    std::vector<int32_t> r, c;
    std::vector<float> v;
    // reserved from the size line, but not trusting it beyond 4 M entries (the vectors grow past that)
    const size_t want = static_cast<size_t>(std::min<long long>(ne, 1LL << 22)) * (mirror ? 2 : 1);
    r.reserve(want);
    c.reserve(want);
    v.reserve(want);
    long long seen = 0;
    while (seen < ne && next_line(fc.f, &fc.line, &cap)) {
        if (fc.line[0] == '%' || blank(fc.line))
            continue;
        char *p = fc.line, *end = nullptr;
        errno = 0;
        const long long i = strtoll(p, &end, 10);
        if (end == p)
            return fail(GCOO_ERROR_INVALID_VALUE, "entry " + std::to_string(seen + 1) + ": no row index");
        p = end;
        const long long j = strtoll(p, &end, 10);
        if (end == p)
            return fail(GCOO_ERROR_INVALID_VALUE, "entry " + std::to_string(seen + 1) + ": no column index");
        p = end;
        float x = 1.0f;
        if (!pattern) {
            const double d = strtod(p, &end);
            if (end == p)
                return fail(GCOO_ERROR_INVALID_VALUE, "entry " + std::to_string(seen + 1) + ": no value");
            x = static_cast<float>(d); // the reference: (float)atof
        }
        if (i < 1 || i > nr || j < 1 || j > nc)
            return fail(GCOO_ERROR_INVALID_VALUE, "entry " + std::to_string(seen + 1) + ": index (" +
                                                      std::to_string(i) + ", " + std::to_string(j) +
                                                      ") outside " + std::to_string(nr) + " x " + std::to_string(nc));
        r.push_back(static_cast<int32_t>(i - 1));
        c.push_back(static_cast<int32_t>(j - 1));
        v.push_back(x);
        if (mirror != 0 && i != j) {
            r.push_back(static_cast<int32_t>(j - 1));
            c.push_back(static_cast<int32_t>(i - 1));
            v.push_back(mirror > 0 ? x : -x);
        }
        ++seen;
    }
    if (seen < ne)
        return fail(GCOO_ERROR_INVALID_VALUE, "the file ends after " + std::to_string(seen) + " of " +
                                                  std::to_string(ne) + " entries");
    while (next_line(fc.f, &fc.line, &cap))
        if (fc.line[0] != '%' && !blank(fc.line))
            return fail(GCOO_ERROR_INVALID_VALUE, "more entries than the size line states");
    if (r.size() > 0x7fffffffULL)
        return fail(GCOO_ERROR_FORMAT, "more triplets than the int32 GCOO format holds");

    const size_t n = r.size();
    int32_t *ro = static_cast<int32_t *>(malloc(std::max<size_t>(n, 1) * sizeof(int32_t)));
    int32_t *co = static_cast<int32_t *>(malloc(std::max<size_t>(n, 1) * sizeof(int32_t)));
    float *vo = static_cast<float *>(malloc(std::max<size_t>(n, 1) * sizeof(float)));
    if (!ro || !co || !vo) {
        free(ro);
        free(co);
        free(vo);
        return fail(GCOO_ERROR_ALLOC, "host allocation of the triplets failed");
    }
    if (n) {
        memcpy(ro, r.data(), n * sizeof(int32_t));
        memcpy(co, c.data(), n * sizeof(int32_t));
        memcpy(vo, v.data(), n * sizeof(float));
    }
    *rows = ro;
    *cols = co;
    *vals = vo;
    *m = nr;
    *k = nc;
    *count = static_cast<int64_t>(n);
    return GCOO_SUCCESS;
}

// fail() builds its message in a std::string: if even that cannot be
// allocated, the status alone is returned.
gcoo_status fail_nothrow(gcoo_status s, const char *msg) noexcept
{
    try {
        return fail(s, msg);
    } catch (...) {
        return s;
    }
}

} // namespace
} // namespace gcoo

using namespace gcoo;

extern "C" {

gcoo_status gcoo_read_matrix_market(const char *path, int64_t *m, int64_t *k, int64_t *count, int32_t **rows,
                                    int32_t **cols, float **vals)
{
    if (!path || !m || !k || !count || !rows || !cols || !vals)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL argument");
    *rows = nullptr;
    *cols = nullptr;
    *vals = nullptr;
    *m = *k = *count = 0;
    try {
        return read_matrix_market(path, m, k, count, rows, cols, vals);
    } catch (const std::bad_alloc &) {
        return fail_nothrow(GCOO_ERROR_ALLOC, "host allocation failed while reading the file");
    } catch (...) {
        return fail_nothrow(GCOO_ERROR_INVALID_VALUE, "the file could not be read");
    }
}

void gcoo_free_host(void *p) { free(p); }

} // extern "C"
