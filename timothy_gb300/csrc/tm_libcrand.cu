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
// M^n S_t.  The host reaches the requested offset by powers of M (squaring);
// on the device, chunk c of kChunk values starts from M^(c kChunk) S, which
// its thread builds from a table of M^(kChunk 2^b) (the bits of c), and one
// thread per chunk runs the recurrence.  The thread of the last chunk leaves
// the window after the last value, so a session's next call continues from
// it without any power on the host.
#include "tm_kernels.cuh"
#include "timothy_gb300.h"

#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

namespace {

constexpr int kWin = 31;
constexpr int kChunk = TM_RAND_CHUNK;   // 31 x 32: a chunk is whole blocks of 31 steps
static_assert(kChunk % kWin == 0, "chunks of whole 31-step blocks");
constexpr int kPowers = 24;   // M^(kChunk 2^b), b < kPowers: up to 2^24 chunks of one call

// the table of jumps, transposed (entry [k * 31 + i] = M[i][k]), copied to
// each device on first use
__device__ uint32_t g_jump[kPowers][kWin * kWin];

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

struct window31 {
    uint32_t w[kWin];
};

// the starting window of every chunk, M^(c kChunk) w0: one warp per chunk,
// lane i holds entry i, and each jump is a matrix-vector product with the
// window broadcast lane by lane
__global__ void __launch_bounds__(128) k_rand_windows(window31 w0, int64_t nchunks, uint32_t *windows)
{
    const int lane = threadIdx.x & 31;
    const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= nchunks) return;                  // whole warp
    uint32_t v = 0u;
#pragma unroll
    for (int i = 0; i < kWin; i++)
        if (lane == i) v = w0.w[i];
    int64_t bits = c;
    for (int b = 0; bits != 0 && b < kPowers; b++, bits >>= 1) {
        if (!(bits & 1)) continue;             // uniform over the warp
        const uint32_t *mt = g_jump[b];
        uint32_t acc = 0u;
#pragma unroll
        for (int k = 0; k < kWin; k++) {
            const uint32_t vk = __shfl_sync(0xffffffffu, v, k);
            if (lane < kWin) acc += __ldg(mt + k * kWin + lane) * vk;
        }
        v = acc;
    }
    if (lane < kWin) windows[c * kWin + lane] = v;
}

// one thread per chunk runs the recurrence in blocks of 31 steps, the window
// in registers: at a block's start w[j] = r[t + j - 31], and step j makes
// r[t + j] = w[j] + (j < 3 ? w[j + 28] : the new w[j - 3]) in place.  The
// last block stops at the stream's end, and its thread writes the window
// after the last value (w from the stop, in stream order).
__global__ void __launch_bounds__(128) k_libc_rand(const uint32_t *windows, int64_t count, int *out, uint32_t *endw)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t first = c * kChunk;
    if (first >= count) return;
    uint32_t w[kWin];
#pragma unroll
    for (int i = 0; i < kWin; i++) w[i] = windows[c * kWin + i];
    const int64_t last = first + kChunk < count ? first + kChunk : count;
    int64_t k0 = first;
    for (; k0 + kWin <= last; k0 += kWin) {
#pragma unroll
        for (int j = 0; j < kWin; j++) {
            w[j] += w[j < 3 ? j + kWin - 3 : j - 3];
            out[k0 + j] = (int)(w[j] >> 1);
        }
    }
    const int rem = (int)(last - k0);          // 0..30 steps of a last, partial block
#pragma unroll
    for (int j = 0; j < kWin; j++) {
        if (j < rem) {
            w[j] += w[j < 3 ? j + kWin - 3 : j - 3];
            out[k0 + j] = (int)(w[j] >> 1);
        }
    }
    if (last == count) {
        // the oldest entry is w[rem] (w[0] after a whole block): rotate by rem
        // as fixed rotations by its bits, so every index stays static
#pragma unroll
        for (int bit = 1; bit < 32; bit <<= 1) {
            if (rem & bit) {
                uint32_t t[kWin];
#pragma unroll
                for (int i = 0; i < kWin; i++) t[i] = w[(i + bit) % kWin];
#pragma unroll
                for (int i = 0; i < kWin; i++) w[i] = t[i];
            }
        }
#pragma unroll
        for (int i = 0; i < kWin; i++) endw[i] = w[i];
    }
}

// the jump table on the current device (once per device and process)
int ensure_jumps()
{
    static std::mutex mtx;
    static bool done[64] = {};
    static std::vector<uint32_t> table;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return -2;
    std::lock_guard<std::mutex> lock(mtx);
    if (done[dev]) return 0;
    if (table.empty()) {
        table.resize((size_t)kPowers * kWin * kWin);
        mat31 m = power(step_matrix(), kChunk);
        for (int b = 0; b < kPowers; b++) {
            uint32_t *t = &table[(size_t)b * kWin * kWin];
            for (int i = 0; i < kWin; i++)
                for (int k = 0; k < kWin; k++) t[k * kWin + i] = m.m[i][k];
            m = mul(m, m);
        }
    }
    if (cudaMemcpyToSymbol(g_jump, table.data(), table.size() * sizeof(uint32_t)) != cudaSuccess) return -2;
    done[dev] = true;
    return 0;
}

}  // namespace

// count values of the stream after srand(seed), starting with the value
// rand() returns after offset earlier calls, into out (device); cache (31
// words + the offset they stand at, host) lets consecutive calls continue
// without the matrix powers
// count values of the stream whose window is w (31 words, oldest first: the
// next value is (w[0] + w[28]) >> 1) into out (device); end receives the
// window after the last value
int tm_libc_rand_from_window(const uint32_t w[31], int64_t count, int *out, uint32_t end[31], uint32_t *d_windows,
                             int64_t windows_cap, cudaStream_t st)
{
    if (count <= 0) {
        memcpy(end, w, kWin * sizeof(uint32_t));
        return 0;
    }
    const int64_t nchunks = (count + kChunk - 1) / kChunk;
    if (nchunks + 1 > windows_cap || nchunks > ((int64_t)1 << kPowers)) return -1;
    if (ensure_jumps() != 0) return -2;
    window31 w0;
    memcpy(w0.w, w, sizeof w0.w);
    uint32_t *endw = d_windows + nchunks * kWin;   // the spare window after the chunks'
    k_rand_windows<<<(unsigned)((nchunks * 32 + 127) / 128), 128, 0, st>>>(w0, nchunks, d_windows);
    const int threads = 128;
    k_libc_rand<<<(unsigned)((nchunks + threads - 1) / threads), threads, 0, st>>>(d_windows, count, out, endw);
    if (cudaGetLastError() != cudaSuccess) return -2;
    if (cudaMemcpyAsync(end, endw, kWin * sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess) return -2;
    if (cudaStreamSynchronize(st) != cudaSuccess) return -2;
    return 0;
}

int tm_libc_rand_device(uint32_t seed, int64_t offset, int64_t count, int *out, tm_rand_cache *cache,
                        uint32_t *d_windows, int64_t windows_cap, cudaStream_t st)
{
    if (count <= 0) return 0;
    window31 w0;
    if (cache && cache->valid && cache->seed == seed && cache->offset == offset) {
        memcpy(w0.w, cache->window, sizeof w0.w);
    } else {
        window_at(seed, (uint64_t)offset, w0.w);
    }
    uint32_t end[kWin];
    const int rc = tm_libc_rand_from_window(w0.w, count, out, end, d_windows, windows_cap, st);
    if (rc != 0) return rc;
    if (cache) {
        memcpy(cache->window, end, sizeof end);
        cache->seed = seed;
        cache->offset = offset + count;
        cache->valid = 1;
    }
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
