// main.cpp -- the -algo benchmark driver with the reference's command line
// (hclhkbu/gcoospdm src/main.cu:180-223) and its output lines
// ("A[..] * B[..]", "Algorithm:", "nnz cpu:", "Time:<microseconds>").
//
//   gcoo_main -nRowsA=800 -nColsA=800 -nRowsB=800 -nColsB=800 -sparsity=0.9 -algo=gcoospdm
//
// As in the reference, "A" is the dense operand (nRowsA x nColsA) and "B" the
// sparse one (nRowsB x nColsB, made sparse by -sparsity); the plugin computes
// C = B x A (nRowsB x nColsA), which needs nColsB == nRowsA.
// Inputs are seeded (-seed, splitmix64 per element: values U(-1,1), never
// exactly zero, Bernoulli mask); the reference used unseeded rand().
// Extensions: -seed, -check=1 (FP64 CPU check, small sizes), -prec=fp32|bf16|
// split|fp8 (with -kernelonly=1), -reps.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "SpGemmBuilder.h"

namespace {

const char *flag_value(int argc, char **argv, const char *name)
{
    const size_t len = strlen(name);
    for (int i = 1; i < argc; ++i) {
        const char *a = argv[i];
        while (*a == '-')
            ++a;
        if (strncmp(a, name, len) == 0 && (a[len] == '=' || a[len] == 0))
            return a[len] == '=' ? a + len + 1 : "";
    }
    return nullptr;
}

uint64_t splitmix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint64_t stream_key(uint64_t seed, uint64_t stream) { return splitmix64(seed + stream * 0xD1B54A32D192ED03ull); }

float pm1(uint64_t h)
{
    const int64_t u = static_cast<int64_t>(h >> 40);
    return static_cast<float>(static_cast<double>(2 * u + 1 - (1LL << 24)) / static_cast<double>(1 << 24));
}

// Same values as gcoospdm_gb300.datagen.bernoulli_dense / dense_pm1.
long long fill(std::vector<float> &x, size_t rows, size_t cols, uint64_t seed, double p, bool sparse)
{
    const uint64_t km = stream_key(seed, 1), kv = stream_key(seed, sparse ? 2 : 5);
    const uint64_t thr = static_cast<uint64_t>(p * 9007199254740992.0);
    long long nnz = 0;
    x.resize(rows * cols);
    for (size_t i = 0; i < rows * cols; ++i) {
        const bool keep = !sparse || (splitmix64(km + i) >> 11) < thr;
        x[i] = keep ? pm1(splitmix64(kv + i)) : 0.0f;
        nnz += keep;
    }
    return nnz;
}

#define CK(call)                                                                          \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            fprintf(stderr, "%s failed: %s\n", #call, cudaGetErrorString(e_));            \
            exit(1);                                                                      \
        }                                                                                 \
    } while (0)

} // namespace

int main(int argc, char **argv)
{
    printf("[Benchmark sparse gemm on GPU (Dense A multiply sparse B] - Starting...\n");
    if (flag_value(argc, argv, "help") || flag_value(argc, argv, "?")) {
        printf("Usage -nRowsA=nRowsA -nColsA=nColsA -nRowsB=nRowsB -nColsB=nColsB\n"
               "      -sparsity=sparsity (of matrix B) -algo=gcoospdm|cublas|cusparse|csr\n"
               "      -kernelonly=0|1 -seed=N -check=0|1 -prec=fp32|bf16|split|fp8 -reps=N\n"
               "      -file=matrix.mtx (Matrix Market; then C = M x M for the file's square M)\n"
               "nColsB should equal nRowsA\n");
        return 0;
    }
    auto geti = [&](const char *n, long long d) {
        const char *v = flag_value(argc, argv, n);
        return v && *v ? atoll(v) : d;
    };
    size_t nRowsA = geti("nRowsA", 1024), nColsA = geti("nColsA", 1024);
    size_t nRowsB = geti("nRowsB", 1024), nColsB = geti("nColsB", 1024);
    const char *sv = flag_value(argc, argv, "sparsity");
    double sparsity = sv && *sv ? atof(sv) : 0.5;
    const char *av = flag_value(argc, argv, "algo");
    std::string algo = av ? av : "gcoospdm";
    bool kernelonly = geti("kernelonly", 0) == 1;
    const uint64_t seed = static_cast<uint64_t>(geti("seed", 1));
    bool check = geti("check", 0) == 1;
    const char *pv = flag_value(argc, argv, "prec");
    std::string prec = pv ? pv : "fp32";
    gcoo_precision gp = GCOO_PREC_FP32;
    if (prec == "bf16") gp = GCOO_PREC_BF16;
    else if (prec == "split") gp = GCOO_PREC_SPLIT_BF16;
    else if (prec == "fp8") gp = GCOO_PREC_FP8_B;

    std::vector<float> A, B;
    long long nnz = 0;
    const char *file = flag_value(argc, argv, "file");
    if (file) {
        // C = M x M for the file's matrix M (src/main.cu:149-176): M is the
        // sparse operand and, densified, the dense one too
        int64_t fm = 0, fk = 0, cnt = 0;
        int32_t *fr = nullptr, *fc = nullptr;
        float *fv = nullptr;
        if (!*file || gcoo_read_matrix_market(file, &fm, &fk, &cnt, &fr, &fc, &fv) != GCOO_SUCCESS) {
            fprintf(stderr, "-file: %s\n", *file ? gcoo_last_error() : "no file name");
            return 2;
        }
        printf("Read mtx file: %s\n", file);
        if (fm != fk) {
            fprintf(stderr, "-file: C = M x M needs a square matrix, got %lld x %lld\n", (long long)fm, (long long)fk);
            gcoo_free_host(fr), gcoo_free_host(fc), gcoo_free_host(fv);
            return 2;
        }
        B.assign(static_cast<size_t>(fm) * static_cast<size_t>(fk), 0.0f);
        for (int64_t i = 0; i < cnt; ++i) // in file order: a later duplicate overwrites, as in the reference
            B[static_cast<size_t>(fr[i]) * static_cast<size_t>(fk) + static_cast<size_t>(fc[i])] = fv[i];
        gcoo_free_host(fr), gcoo_free_host(fc), gcoo_free_host(fv);
        A = B;
        nRowsA = nColsA = nRowsB = nColsB = static_cast<size_t>(fm);
        for (float x : B)
            nnz += x != 0.0f;
    } else {
        if (nColsB != nRowsA) {
            fprintf(stderr, "nColsB (%zu) must equal nRowsA (%zu)\n", nColsB, nRowsA);
            return 2;
        }
        fill(A, nRowsA, nColsA, seed, 1.0, false);
        nnz = fill(B, nRowsB, nColsB, seed, 1.0 - sparsity, true);
    }
    printf("nnz cpu: %lld, density: %.4f\n", nnz, nnz * 1.0 / (double)(nRowsB * nColsB));
    printf("A[%zu,%zu] * B[%zu,%zu]\n", nRowsA, nColsA, nRowsB, nColsB);
    printf("Algorithm: %s\n", algo.c_str());

    const size_t m = nRowsB, k = nColsB, n = nColsA;
    float *dA = nullptr, *dB = nullptr, *dC = nullptr;
    CK(cudaMalloc(&dA, A.size() * sizeof(float)));
    CK(cudaMalloc(&dB, B.size() * sizeof(float)));
    CK(cudaMalloc(&dC, m * n * sizeof(float)));
    CK(cudaMemcpy(dA, A.data(), A.size() * sizeof(float), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(dB, B.data(), B.size() * sizeof(float), cudaMemcpyHostToDevice));

    ShGemm *g = SpGemmBuilder::getShGemmAlgo(dB, (int)nRowsB, (int)nColsB, algo);
    if (!g) {
        fprintf(stderr, "unknown -algo=%s (supported: gcoospdm, cublas, cusparse, csr)\n", algo.c_str());
        return 2;
    }
    ShGCOOSpDM *gc = algo == "gcoospdm" ? static_cast<ShGCOOSpDM *>(g) : nullptr;
    int reps = (int)geti("reps", nRowsA > 8000 ? 20 : 100); // src/main.cu:46-49
    auto call = [&]() -> double {
        if (!kernelonly)
            return g->mutiplyBy(dA, (int)nRowsA, (int)nColsA, dC);
        if (gc && gp != GCOO_PREC_FP32)
            return gc->runKernelTest(dA, (int)nRowsA, (int)nColsA, dC, gp);
        return g->runKernelTest(dA, (int)nRowsA, (int)nColsA, dC);
    };
    if (kernelonly)
        g->build();
    if (call() < 0) { // warm-up
        fprintf(stderr, "the first call failed\n");
        return 1;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, 0);
    for (int i = 0; i < reps; ++i)
        if (call() < 0) {
            fprintf(stderr, "call %d failed\n", i);
            return 1;
        }
    cudaEventRecord(e1, 0);
    CK(cudaEventSynchronize(e1));
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    ms /= reps;
    std::vector<float> C(m * n);
    CK(cudaMemcpy(C.data(), dC, C.size() * sizeof(float), cudaMemcpyDeviceToHost));
    printf("Time:%f\n", ms * 1000.0f);
    printf("GFLOPS:%f\n", 2.0 * (double)nnz * (double)n / (ms * 1e6));
    int rc = 0;
    if (check) {
        double num = 0.0, den = 0.0;
        for (size_t r = 0; r < m; ++r)
            for (size_t j = 0; j < n; ++j) {
                double s = 0.0;
                for (size_t c = 0; c < k; ++c)
                    s += (double)B[r * k + c] * (double)A[c * n + j];
                const double d = (double)C[r * n + j] - s;
                num += d * d;
                den += s * s;
            }
        const double rel = den > 0 ? sqrt(num / den) : sqrt(num);
        printf("RelFrobenius:%e\n", rel);
        const double tol = gp == GCOO_PREC_FP32 || gp == GCOO_PREC_SPLIT_BF16 ? 1e-5 : (gp == GCOO_PREC_BF16 ? 1e-2 : 5e-2);
        if (rel <= tol)
            printf("Test passed\n");
        else {
            printf("Test failed\n");
            rc = 1;
        }
    }
    delete g;
    cudaFree(dA);
    cudaFree(dB);
    cudaFree(dC);
    return rc;
}
