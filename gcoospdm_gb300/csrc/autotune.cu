// autotune.cu -- runtime autotuner replacing the reference's template
// regeneration + recompile loop (src/autotune.py:45-103 over
// src/constants.h.t's $COLUMN_PER_GROUP$ / $BS$). Launch shapes are runtime
// parameters here, so a candidate is timed with CUDA events on the caller's
// stream instead of rebuilt; the winner is stored in an in-process table
// keyed by shape bucket and can be saved to / loaded from a small JSON file.
//
// Bucket of a multiply: ceil(log2 m), ceil(log2 k), floor(-log2 density),
// ceil(log2 n). Batched plans store their per-bucket rows-per-work-item
// choice in the same table (see batched.cu).
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "handle.hpp"

namespace gcoo {

static std::mutex g_tune_mu;
static std::map<std::string, TuneEntry> g_table;

static int clog2(int64_t x)
{
    int r = 0;
    while ((int64_t(1) << r) < x)
        ++r;
    return r;
}

std::string bucket_key(int64_t m, int64_t k, int64_t nnz, int64_t n)
{
    const double density = (m > 0 && k > 0) ? static_cast<double>(nnz) / (static_cast<double>(m) * k) : 0.0;
    const int d = density > 0.0 ? static_cast<int>(floor(-log2(density))) : 99;
    char buf[96];
    snprintf(buf, sizeof buf, "m%d_k%d_d%d_n%d", clog2(m), clog2(k), d, clog2(n));
    return buf;
}

bool tune_lookup(const std::string &key, TuneEntry *out)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_table.find(key);
    if (it == g_table.end())
        return false;
    *out = it->second;
    return true;
}

void tune_store(const std::string &key, const TuneEntry &e)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_table[key] = e;
}

bool tuned_params(int64_t m, int64_t k, int64_t nnz, int64_t n, gcoo_params *out)
{
    TuneEntry e;
    if (!tune_lookup(bucket_key(m, k, nnz, n), &e) || e.vec == 0)
        return false;
    out->vec = e.vec;
    out->warps = e.warps;
    out->col_warps = e.col_warps;
    out->depth = e.depth;
    return true;
}

gcoo_status spdm_fp32(gcoo_handle *h, const float *dB, int64_t n, float *dC, cudaStream_t st,
                      const gcoo_params *override_params);

} // namespace gcoo

using namespace gcoo;

extern "C" {

gcoo_status gcoo_autotune(gcoo_handle *h, const float *dB, int64_t n, float *dC, void *stream, gcoo_params *best)
{
    if (!h || !dB || !dC)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL argument");
    if (!h->built)
        return fail(GCOO_ERROR_NOT_BUILT, "gcoo_build has not run");
    if (n <= 0 || n >= (int64_t(1) << 31))
        return fail(GCOO_ERROR_INVALID_VALUE, "n must be in [1, 2^31)");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0, e1;
    GCOO_CUDA(cudaEventCreate(&e0));
    GCOO_CUDA(cudaEventCreate(&e1));
    const int cpg = h->p.rows_per_group;
    std::vector<gcoo_params> cands;
    for (int vec : {1, 2, 4}) {
        for (int warps : {4, 8, 16, 32}) {
            for (int depth : {1, 2}) {
                if (warps < cpg)
                    continue;
                gcoo_params p = h->p;
                p.vec = vec;
                p.warps = warps;
                p.col_warps = 0;
                p.depth = depth;
                cands.push_back(p);
            }
        }
    }
    double best_us = 1e30;
    gcoo_params best_p = h->p;
    LaunchShape best_shape{};
    for (const gcoo_params &p : cands) {
        const LaunchShape s = pick_shape(p, h->m, n, h->nnz, h->max_row_nnz, reinterpret_cast<uintptr_t>(dB),
                                         reinterpret_cast<uintptr_t>(dC));
        if (s.vec != p.vec)
            continue; // not valid for this width / alignment
        gcoo_status r = spdm_fp32(h, dB, n, dC, st, &p); // warm-up
        if (r != GCOO_SUCCESS)
            continue;
        float ms_best = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            cudaEventRecord(e0, st);
            spdm_fp32(h, dB, n, dC, st, &p);
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < ms_best)
                ms_best = ms;
        }
        if (ms_best * 1e3 < best_us) {
            best_us = ms_best * 1e3;
            best_p = p;
            best_shape = s;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    GCOO_CUDA(cudaGetLastError());
    if (best_us >= 1e30)
        return fail(GCOO_ERROR_UNSUPPORTED, "no candidate launch shape is valid");
    TuneEntry e;
    e.vec = best_shape.vec;
    e.warps = best_shape.warps;
    e.col_warps = best_shape.col_warps;
    e.depth = best_shape.depth;
    e.us = best_us;
    tune_store(bucket_key(h->m, h->k, h->nnz, n), e);
    if (best) {
        *best = best_p;
        best->vec = e.vec;
        best->warps = e.warps;
        best->col_warps = e.col_warps;
        best->depth = e.depth;
    }
    return GCOO_SUCCESS;
}

gcoo_status gcoo_autotune_save(const char *path)
{
    if (!path)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL path");
    FILE *f = fopen(path, "w");
    if (!f)
        return fail(GCOO_ERROR_INVALID_VALUE, std::string("cannot write ") + path);
    std::lock_guard<std::mutex> lock(g_tune_mu);
    fprintf(f, "{\"version\": 1, \"entries\": [\n");
    size_t i = 0;
    for (const auto &kv : g_table) {
        const TuneEntry &e = kv.second;
        fprintf(f, "{\"bucket\": \"%s\", \"vec\": %d, \"warps\": %d, \"col_warps\": %d, \"depth\": %d, \"rows_per_item\": %d, \"us\": %.3f}%s\n",
                kv.first.c_str(), e.vec, e.warps, e.col_warps, e.depth, e.rows_per_item, e.us, ++i < g_table.size() ? "," : "");
    }
    fprintf(f, "]}\n");
    fclose(f);
    return GCOO_SUCCESS;
}

gcoo_status gcoo_autotune_load(const char *path)
{
    if (!path)
        return fail(GCOO_ERROR_INVALID_VALUE, "NULL path");
    FILE *f = fopen(path, "r");
    if (!f)
        return fail(GCOO_ERROR_INVALID_VALUE, std::string("cannot read ") + path);
    char line[512];
    int loaded = 0;
    while (fgets(line, sizeof line, f)) {
        char bucket[128];
        TuneEntry e;
        if (sscanf(line, " {\"bucket\": \"%127[^\"]\", \"vec\": %d, \"warps\": %d, \"col_warps\": %d, \"depth\": %d, \"rows_per_item\": %d, \"us\": %lf",
                   bucket, &e.vec, &e.warps, &e.col_warps, &e.depth, &e.rows_per_item, &e.us) == 7) {
            tune_store(bucket, e);
            ++loaded;
        }
    }
    fclose(f);
    return loaded > 0 ? GCOO_SUCCESS : fail(GCOO_ERROR_INVALID_VALUE, std::string("no entries in ") + path);
}

gcoo_status gcoo_autotune_clear(void)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_table.clear();
    return GCOO_SUCCESS;
}

} // extern "C"
