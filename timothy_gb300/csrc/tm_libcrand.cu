// The C library's rand() stream after srand(seed), generated on the device.
//
// The stream is glibc's random() with its default state (TYPE_3): 34 words
// seeded by the multiplicative generator r[i] = 16807 r[i-1] mod (2^31 - 1)
// (Schrage's factorisation, so no intermediate overflows), r[31..33] copies
// of r[0..2], then r[i] = r[i-31] + r[i-3] mod 2^32; the first 310 values of
// that recurrence are discarded, and the k-th value returned is
// r[344 + k] >> 1.  (The published description of the generator; the
// reference draws its cell-cycle decisions from it in cell order.)
//
// The recurrence is linear over the integers mod 2^32, so the window
// S_t = (r[t-31], ..., r[t-1]) advances by a 31 x 31 matrix M: S_{t+n} =
// M^n S_t.  The host reaches the requested offset by powers of M (squaring),
// then gives each of the chunks of kChunk values its starting window by
// repeated multiplication with M^kChunk; one device thread per chunk runs
// the recurrence.  A session remembers where its last stream ended, so
// consecutive calls continue without the powers.
#include "tm_kernels.cuh"
#include "timothy_gb300.h"

#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr int kWin = 31;
constexpr int kChunk = 2048;

struct mat31 {
    uint32_t m[kWin][kWin];
};

// S_{t+1} = M S_t: the new last entry is r[t-31] + r[t-3], the rest shift
mat31 step_matrix()
{
    mat31 a;
    memset(&a, 0, sizeof a);
    for (int r = 0; r + 1 < kWin; r++) a.m[r][r + 1] = 1u;
    a.m[kWin - 1][0] = 1u;
    a.m[kWin - 1][kWin - 3] += 1u;
    return a;
}

mat31 mul(const mat31 &x, const mat31 &y)
{
    mat31 z;
    for (int i = 0; i < kWin; i++)
        for (int j = 0; j < kWin; j++) {
            uint32_t s = 0;
            for (int k = 0; k < kWin; k++) s += x.m[i][k] * y.m[k][j];
            z.m[i][j] = s;
        }
    return z;
}

void apply(const mat31 &x, const uint32_t in[kWin], uint32_t out[kWin])
{
    for (int i = 0; i < kWin; i++) {
        uint32_t s = 0;
        for (int k = 0; k < kWin; k++) s += x.m[i][k] * in[k];
        out[i] = s;
    }
}

mat31 power(mat31 base, uint64_t n)
{
    mat31 r;
    memset(&r, 0, sizeof r);
    for (int i = 0; i < kWin; i++) r.m[i][i] = 1u;
    while (n) {
        if (n & 1u) r = mul(r, base);
        base = mul(base, base);
        n >>= 1;
    }
    return r;
}

// the window S_t at t = 344 + offset (the next value returned is r[t] >> 1)
void window_at(uint32_t seed, uint64_t offset, uint32_t w[kWin])
{
    uint32_t r[34];
    int32_t word = (int32_t)(seed == 0 ? 1u : seed);
    r[0] = (uint32_t)word;
    for (int i = 1; i < 31; i++) {
        const int64_t hi = word / 127773, lo = word % 127773;
        int64_t v = 16807 * lo - 2836 * hi;
        if (v < 0) v += 2147483647;
        word = (int32_t)v;
        r[i] = (uint32_t)word;
    }
    for (int i = 31; i < 34; i++) r[i] = r[i - 31];
    // S_34 = (r[3], ..., r[33])
    uint32_t s[kWin];
    for (int i = 0; i < kWin; i++) s[i] = r[3 + i];
    const uint64_t n = 310 + offset;      // to t = 344 + offset
    if (n < 4096) {
        for (uint64_t k = 0; k < n; k++) {
            const uint32_t v = s[0] + s[kWin - 3];
            memmove(s, s + 1, (kWin - 1) * sizeof(uint32_t));
            s[kWin - 1] = v;
        }
        memcpy(w, s, sizeof s);
    } else {
        apply(power(step_matrix(), n), s, w);
    }
}

__global__ void k_libc_rand(const uint32_t *windows, int64_t count, int *out)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t first = c * kChunk;
    if (first >= count) return;
    uint32_t w[kWin];
    for (int i = 0; i < kWin; i++) w[i] = windows[c * kWin + i];
    const int64_t last = first + kChunk < count ? first + kChunk : count;
    int head = 0;                          // w[head] is the oldest entry, r[t-31]
    for (int64_t k = first; k < last; k++) {
        int i3 = head + kWin - 3;
        if (i3 >= kWin) i3 -= kWin;
        const uint32_t v = w[head] + w[i3];
        w[head] = v;
        head = head + 1 == kWin ? 0 : head + 1;
        out[k] = (int)(v >> 1);
    }
}

}  // namespace

// count values of the stream after srand(seed), starting with the value
// rand() returns after offset earlier calls, into out (device); cache (31
// words + the offset they stand at, host) lets consecutive calls continue
// without the matrix powers
int tm_libc_rand_device(uint32_t seed, int64_t offset, int64_t count, int *out, tm_rand_cache *cache,
                        uint32_t *d_windows, int64_t windows_cap, cudaStream_t st)
{
    if (count <= 0) return 0;
    const int64_t nchunks = (count + kChunk - 1) / kChunk;
    if (nchunks > windows_cap) return -1;
    uint32_t w[kWin];
    if (cache && cache->valid && cache->seed == seed && cache->offset == offset) {
        memcpy(w, cache->window, sizeof w);
    } else {
        window_at(seed, (uint64_t)offset, w);
    }
    std::vector<uint32_t> win((size_t)nchunks * kWin);
    static const mat31 jump = power(step_matrix(), kChunk);
    memcpy(win.data(), w, sizeof w);
    for (int64_t c = 1; c < nchunks; c++) apply(jump, &win[(size_t)(c - 1) * kWin], &win[(size_t)c * kWin]);
    // the window after the last value, for the next call
    if (cache) {
        uint32_t endw[kWin];
        const int64_t rest = count - (nchunks - 1) * kChunk;
        apply(power(step_matrix(), (uint64_t)rest), &win[(size_t)(nchunks - 1) * kWin], endw);
        memcpy(cache->window, endw, sizeof endw);
        cache->seed = seed;
        cache->offset = offset + count;
        cache->valid = 1;
    }
    if (cudaMemcpyAsync(d_windows, win.data(), win.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st) !=
        cudaSuccess)
        return -2;
    const int threads = 128;
    k_libc_rand<<<(unsigned)((nchunks + threads - 1) / threads), threads, 0, st>>>(d_windows, count, out);
    if (cudaGetLastError() != cudaSuccess) return -2;
    // the host vector must outlive the copy
    if (cudaStreamSynchronize(st) != cudaSuccess) return -2;
    return 0;
}

// the same values computed on the host, chunk by chunk as the device does
// (for tests of the stream against the C library)
extern "C" int tmi_libc_rand_host(uint32_t seed, int64_t offset, int64_t count, int *out)
{
    if (count <= 0) return TM_OK;
    uint32_t w[kWin];
    window_at(seed, (uint64_t)offset, w);
    static const mat31 jump = power(step_matrix(), kChunk);
    for (int64_t first = 0; first < count; first += kChunk) {
        uint32_t s[kWin];
        memcpy(s, w, sizeof s);
        const int64_t last = first + kChunk < count ? first + kChunk : count;
        for (int64_t k = first; k < last; k++) {
            const uint32_t v = s[0] + s[kWin - 3];
            memmove(s, s + 1, (kWin - 1) * sizeof(uint32_t));
            s[kWin - 1] = v;
            out[k] = (int)(v >> 1);
        }
        uint32_t nw[kWin];
        apply(jump, w, nw);
        memcpy(w, nw, sizeof w);
    }
    return TM_OK;
}
