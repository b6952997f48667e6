// mt19937.cu -- Mersenne Twister MT19937 streams for McICA (irng = 1) at
// scale, generated by many CTAs at once through jump-ahead.
//
// The generator is the reference's (mcica_random_numbers.f90:77-306):
// init_genrand from a 32-bit seed, 624-word state, tempering, and
// getRandomReal = u32 / (2^32 - 1).  mcica_subcol_gen_sw.f90 draws one stream
// of length 112*ncol*nlay (x2 for icld 4/5, 112*ncol for icld 3) in
// (subcolumn, column, layer) order, so the draws of one column depend on
// ncol; the single-CTA generator needed ~1 s at 262 144 columns x 60 layers.
//
// Jump-ahead (F2-linear generators; Haramoto, Matsumoto, Nishimura,
// Panneton, L'Ecuyer 2008): with raw words x_k (x_0..x_623 from the seed,
// x_{k+624} = x_{k+397} ^ twist(x_k, x_{k+1})), every bit of x_{m+1} is a
// linear form of the 19937-bit state at time m, whose transition T has a
// characteristic polynomial phi of degree 19937.  If g = x^J mod phi then
// x_{m+J} = XOR over {i : g_i = 1} of x_{m+i} for every m >= 1, so the 624
// words at position m+J come from the 19937+623 words after position m.
// phi is found once on the host by Berlekamp-Massey over 2*19937 output
// bits (it is primitive, so one bit sequence has it as minimal polynomial);
// the table x^(2^b) mod phi, b < 48, follows by repeated squaring.  Segment
// p of length S = 2^s starts at output p*S: one CTA of k_mt_windows composes
// the jumps of the set bits of p (x^(2^(b+s))) into the segment's first 624
// words, then one CTA of k_mt_generate (8 per SM) runs the recurrence over
// the rest of the segment as the sequential generator would.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "launch.h"

namespace rrsw {
namespace mt {

constexpr int NW = 624, MW = 397, DEG = 19937;
constexpr int PW = 312;              // 64-bit words of a reduced polynomial (degree < 19937)
constexpr int EXT = DEG + NW - 1;    // words one jump reads: 20560
constexpr int MAXB = 48;             // jump table x^(2^b) mod phi, b < MAXB
constexpr int WTHREADS = 256;        // window kernel: >= 227 (one recurrence step), >= 156 (jump outputs / 4)
constexpr int GTHREADS = 256;        // generation kernel: >= 227
constexpr uint64_t RING = 1023;      // generation ring: 1024 words, index mask

__host__ __device__ inline uint32_t twist(uint32_t u, uint32_t v) {
    const uint32_t mix = (u & 0x80000000u) | (v & 0x7fffffffu);
    return (mix >> 1) ^ ((v & 1u) ? 0x9908b0dfu : 0u);
}

__host__ __device__ inline uint32_t temper(uint32_t y) {
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
}

// ----------------------------------------------------------------- host side
namespace {

// x_624..x_1247: the state after the first regeneration (the words behind
// outputs 0..623)
void first_window(uint32_t seed, uint32_t* x) {
    std::vector<uint32_t> e(2 * NW);
    e[0] = seed;
    for (int i = 1; i < NW; ++i) e[i] = 1812433253u * (e[i - 1] ^ (e[i - 1] >> 30)) + (uint32_t)i;
    for (int k = NW; k < 2 * NW; ++k) e[k] = e[k - NW + MW] ^ twist(e[k - NW], e[k - NW + 1]);
    std::memcpy(x, e.data() + NW, NW * sizeof(uint32_t));
}

// e[0..623] given; e[624..n) by the recurrence
void extend(uint32_t* e, int n) {
    for (int k = NW; k < n; ++k) e[k] = e[k - NW + MW] ^ twist(e[k - NW], e[k - NW + 1]);
}

inline int bit(const std::vector<uint64_t>& v, long i) { return (int)((v[(size_t)i >> 6] >> (i & 63)) & 1u); }

struct Tables {
    bool ok = false;
    std::vector<uint64_t> phi;      // PW + 1 words, degree DEG
    std::vector<uint64_t> jump;     // MAXB x PW: x^(2^b) mod phi
};

// 64-bit word of v starting at bit pos (bits past the end read 0)
inline uint64_t word_at(const std::vector<uint64_t>& v, size_t pos) {
    const size_t w = pos >> 6;
    const unsigned o = (unsigned)(pos & 63);
    const uint64_t lo = w < v.size() ? v[w] : 0ull;
    if (!o) return lo;
    const uint64_t hi = w + 1 < v.size() ? v[w + 1] : 0ull;
    return (lo >> o) | (hi << (64 - o));
}

inline int parity64(uint64_t x) {
    x ^= x >> 32;
    x ^= x >> 16;
    x ^= x >> 8;
    x ^= x >> 4;
    x ^= x >> 2;
    x ^= x >> 1;
    return (int)(x & 1u);
}

// characteristic polynomial of the MT19937 transition: Berlekamp-Massey
// over GF(2) on the lowest bit of 2*DEG consecutive raw words
bool charpoly(std::vector<uint64_t>& phi) {
    const long n = 2L * DEG;
    std::vector<uint32_t> e(NW + n);
    first_window(5489u, e.data());
    extend(e.data(), (int)e.size());
    const size_t nw = (size_t)(n + 127) / 64;
    std::vector<uint64_t> rev(nw, 0ull);  // bit k = s[n-1-k]
    for (long k = 0; k < n; ++k)
        if (e[n - 1 - k] & 1u) rev[(size_t)k >> 6] |= 1ull << (k & 63);
    std::vector<uint64_t> C(nw, 0ull), B(nw, 0ull), T;
    C[0] = B[0] = 1ull;
    long L = 0, m = 1, degC = 0, degB = 0;
    for (long i = 0; i < n; ++i) {
        // discrepancy: sum_{j=0..L} C_j s[i-j], s[i-j] = bit (n-1-i)+j of rev
        const size_t sh = (size_t)(n - 1 - i);
        uint64_t acc = 0;
        for (long w = 0; w <= degC / 64; ++w) acc ^= C[(size_t)w] & word_at(rev, sh + 64 * (size_t)w);
        if (!parity64(acc)) {
            ++m;
            continue;
        }
        const bool grow = 2 * L <= i;
        if (grow) T = C;
        // C += x^m B
        const long ws = m / 64;
        const unsigned bs = (unsigned)(m % 64);
        for (long w = degB / 64; w >= 0; --w) {
            const uint64_t b = B[(size_t)w];
            if (!b) continue;
            C[(size_t)(w + ws)] ^= b << bs;
            if (bs && (size_t)(w + ws + 1) < nw) C[(size_t)(w + ws + 1)] ^= b >> (64 - bs);
        }
        const long degC_old = degC;
        degC = degC > degB + m ? degC : degB + m;
        if (grow) {
            const long Lnew = i + 1 - L;
            L = Lnew;
            B.swap(T);
            degB = degC_old;
            m = 1;
        } else {
            ++m;
        }
    }
    if (L != DEG) return false;
    // phi(x) = x^L C(1/x): phi_k = C_{L-k}
    phi.assign(PW + 1, 0ull);
    for (long k = 0; k <= L; ++k)
        if (bit(C, L - k)) phi[(size_t)k >> 6] |= 1ull << (k & 63);
    return bit(phi, DEG) == 1;
}

// a^2 mod phi for a reduced polynomial a (PW words)
void sqrmod(const std::vector<uint64_t>& a, const std::vector<std::vector<uint64_t>>& phish,
            std::vector<uint64_t>& out) {
    std::vector<uint64_t> t(2 * PW + 2, 0ull);
    for (int w = 0; w < PW; ++w) {
        const uint64_t x = a[(size_t)w];
        uint64_t lo = 0, hi = 0;
        for (int b = 0; b < 32; ++b) {
            lo |= ((x >> b) & 1ull) << (2 * b);
            hi |= ((x >> (b + 32)) & 1ull) << (2 * b);
        }
        t[(size_t)2 * w] = lo;
        t[(size_t)2 * w + 1] = hi;
    }
    for (long d = 2L * (DEG - 1); d >= DEG; --d) {
        if (!bit(t, d)) continue;
        const long k = d - DEG;
        const std::vector<uint64_t>& ps = phish[(size_t)(k & 63)];
        const size_t off = (size_t)(k >> 6);
        for (size_t w = 0; w < ps.size() && off + w < t.size(); ++w) t[off + w] ^= ps[w];
    }
    out.assign(t.begin(), t.begin() + PW);
}

Tables build_tables() {
    Tables T;
    if (!charpoly(T.phi)) return T;
    std::vector<std::vector<uint64_t>> phish(64);
    for (int r = 0; r < 64; ++r) {
        std::vector<uint64_t>& v = phish[(size_t)r];
        v.assign(PW + 2, 0ull);
        for (int w = 0; w <= PW; ++w) {
            v[(size_t)w] ^= T.phi[(size_t)w] << r;
            if (r) v[(size_t)w + 1] ^= T.phi[(size_t)w] >> (64 - r);
        }
    }
    T.jump.assign((size_t)MAXB * PW, 0ull);
    std::vector<uint64_t> cur(PW, 0ull), nxt;
    cur[0] = 2ull;  // x
    for (int b = 0; b < MAXB; ++b) {
        std::copy(cur.begin(), cur.end(), T.jump.begin() + (size_t)b * PW);
        if (b + 1 < MAXB) {
            sqrmod(cur, phish, nxt);
            cur.swap(nxt);
        }
    }
    // reduced polynomials stop at bit DEG-1
    for (int b = 0; b < MAXB; ++b)
        if (T.jump[(size_t)b * PW + PW - 1] >> (DEG - 64 * (PW - 1))) return Tables{};
    T.ok = true;
    return T;
}

std::mutex g_mu;

const Tables& tables() {
    static Tables T;
    static bool built = false;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!built) {
        T = build_tables();
        built = true;
    }
    return T;
}

// window <- the 624 words J steps later, J = 2^b
void apply_host(uint32_t* win, const uint64_t* g) {
    std::vector<uint32_t> e(EXT);
    std::memcpy(e.data(), win, NW * sizeof(uint32_t));
    extend(e.data(), EXT);
    std::vector<uint32_t> acc(NW, 0u);
    for (int w = 0; w < PW; ++w) {
        uint64_t gw = g[w];
        while (gw) {
            int b = 0;
            while (!((gw >> b) & 1ull)) ++b;
            gw &= gw - 1;
            const uint32_t* src = e.data() + 64 * w + b;
            for (int j = 0; j < NW; ++j) acc[(size_t)j] ^= src[j];
        }
    }
    std::memcpy(win, acc.data(), NW * sizeof(uint32_t));
}

struct DeviceTable {
    int device = -1;
    uint64_t* p = nullptr;
};

std::vector<DeviceTable> g_dev;

cudaError_t device_table(const Tables& T, const uint64_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(g_mu);
    for (const DeviceTable& d : g_dev)
        if (d.device == dev) {
            *out = d.p;
            return cudaSuccess;
        }
    DeviceTable d;
    d.device = dev;
    const size_t bytes = T.jump.size() * sizeof(uint64_t);
    if ((e = cudaMalloc(&d.p, bytes)) != cudaSuccess) return e;
    if ((e = cudaMemcpy(d.p, T.jump.data(), bytes, cudaMemcpyHostToDevice)) != cudaSuccess) {
        cudaFree(d.p);
        return e;
    }
    g_dev.push_back(d);
    *out = d.p;
    return cudaSuccess;
}

}  // namespace

// --------------------------------------------------------------- device side

// In-place regeneration of the 624-word state (three dependency-free
// phases of 227, 227 and 169 words, then the last word).  Starts with a
// read phase and a barrier, so the previous block's readers are done
// before any word is overwritten.
__device__ inline void regenerate(uint32_t* e, int t) {
    uint32_t v = 0;
    if (t < NW - MW) v = e[t + MW] ^ twist(e[t], e[t + 1]);
    __syncthreads();
    if (t < NW - MW) e[t] = v;
    __syncthreads();
    if (t < NW - MW) v = e[t] ^ twist(e[t + 227], e[t + 228]);
    __syncthreads();
    if (t < NW - MW) e[t + 227] = v;
    __syncthreads();
    if (t < 169) v = e[t + 227] ^ twist(e[t + 454], e[t + 455]);
    __syncthreads();
    if (t < 169) e[t + 454] = v;
    __syncthreads();
    if (t == 0) e[NW - 1] = e[MW - 1] ^ twist(e[NW - 1], e[0]);
    __syncthreads();
}

// Kernel 1: the window of segment p = blockIdx.x (the 624 raw words behind
// outputs p*2^logS ..), written raw into the first min(624, len) words of
// the segment's own output range.  Jumps: one per set bit of p; in a jump,
// thread t < 156 forms output words t, t+156, t+312, t+468 so the bit scan
// of the polynomial is shared by four accumulators.
__global__ void __launch_bounds__(WTHREADS) k_mt_windows(uint32_t seed, uint64_t n, int logS,
                                                        const uint64_t* __restrict__ jump,
                                                        uint32_t* __restrict__ out) {
    extern __shared__ __align__(16) uint64_t sm_mt[];
    uint64_t* sp = sm_mt;                      // jump polynomial, PW words
    uint32_t* e = (uint32_t*)(sm_mt + PW);     // EXT words
    const int t = threadIdx.x;
    const uint64_t p = blockIdx.x;
    const uint64_t start = p << logS;
    if (start >= n) return;
    if (t == 0) {
        e[0] = seed;
        for (int i = 1; i < NW; ++i) e[i] = 1812433253u * (e[i - 1] ^ (e[i - 1] >> 30)) + (uint32_t)i;
    }
    __syncthreads();
    regenerate(e, t);  // x_624..x_1247: outputs 0..623
    constexpr int Q = NW / 4;
    for (int b = 0; (p >> b) != 0ull; ++b) {
        if (!((p >> b) & 1ull)) continue;
        const uint64_t* g = jump + (size_t)(b + logS) * PW;
        for (int w = t; w < PW; w += WTHREADS) sp[w] = g[w];
        // the 19936 + 624 words after the window
        for (int q = NW; q < EXT; q += NW - MW) {
            const int k = q + t;
            if (t < NW - MW && k < EXT) e[k] = e[k - NW + MW] ^ twist(e[k - NW], e[k - NW + 1]);
            __syncthreads();
        }
        uint32_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        if (t < Q) {
            for (int w = 0; w < PW; ++w) {
                uint64_t gw = sp[w];
                const uint32_t* ew = e + 64 * w + t;
                while (gw) {
                    const uint32_t* x = ew + (__ffsll((long long)gw) - 1);
                    gw &= gw - 1;
                    a0 ^= x[0];
                    a1 ^= x[Q];
                    a2 ^= x[2 * Q];
                    a3 ^= x[3 * Q];
                }
            }
        }
        __syncthreads();
        if (t < Q) {
            e[t] = a0;
            e[t + Q] = a1;
            e[t + 2 * Q] = a2;
            e[t + 3 * Q] = a3;
        }
        __syncthreads();
    }
    const uint64_t len = (n - start) < (1ull << logS) ? (n - start) : (1ull << logS);
    for (int k = t; k < NW && (uint64_t)k < len; k += WTHREADS) out[start + (uint64_t)k] = e[k];
}

// Kernel 2: segment p from its window, 227 words per step through a
// 1024-word ring (a step writes the slots of words k-1024, which no thread
// of the step reads: reads reach back 624 words), tempered into out.
__global__ void __launch_bounds__(GTHREADS) k_mt_generate(uint64_t n, int logS, uint32_t* __restrict__ out) {
    __shared__ uint32_t ring[RING + 1];
    const int t = threadIdx.x;
    const uint64_t start = (uint64_t)blockIdx.x << logS;
    if (start >= n) return;
    const uint64_t len = (n - start) < (1ull << logS) ? (n - start) : (1ull << logS);
    const int w0 = len < (uint64_t)NW ? (int)len : NW;
    for (int k = t; k < w0; k += GTHREADS) ring[k] = out[start + (uint64_t)k];
    __syncthreads();
    for (int k = t; k < w0; k += GTHREADS) out[start + (uint64_t)k] = temper(ring[k]);
    for (uint64_t k0 = NW; k0 < len; k0 += NW - MW) {
        if (t < NW - MW) {
            const uint64_t k = k0 + (uint64_t)t;
            const uint32_t y =
                ring[(k - (NW - MW)) & RING] ^ twist(ring[(k - NW) & RING], ring[(k - NW + 1) & RING]);
            ring[k & RING] = y;
            if (k < len) out[start + k] = temper(y);
        }
        __syncthreads();
    }
}

}  // namespace mt

size_t mt_jump_smem() { return mt::PW * sizeof(uint64_t) + (size_t)mt::EXT * sizeof(uint32_t); }

// Segment length 2^logS for n words: the windows cost one jump per set
// bit of the segment index (bits below 2^15 are sparse shifts), the
// generation one ring step per 227 words; both modelled in SM cycles.
static int choose_log_seg(uint64_t n, int num_sms) {
    const double sms = num_sms > 0 ? num_sms : 1;
    const double jump_cycles = 2.0e5, gen_sm_rate = 3.0, gen_cta_rate = 0.9;  // words per cycle
    double best = -1.0;
    int pick = 12;
    for (int ls = 12; ls <= 40; ++ls) {
        const uint64_t ns = (n + (1ull << ls) - 1) >> ls;
        const double per_sm = std::ceil((double)ns / sms);
        const double resident = per_sm < 8.0 ? per_sm : 8.0;
        const double rate = std::fmin(gen_cta_rate, gen_sm_rate / resident);
        const double waves = std::ceil((double)ns / (8.0 * sms));
        double dense = 0.0;  // set bits of the segment indices that are dense jumps
        for (int b = 0; (ns - 1) >> b; ++b)
            if (b + ls >= 15) dense += (double)ns / 2.0;
        const double cost = waves * (double)(1ull << ls) / rate + dense * jump_cycles / (2.0 * sms);
        if (best < 0.0 || cost < best) {
            best = cost;
            pick = ls;
        }
        if (ns == 1) break;
    }
    return pick;
}

cudaError_t launch_mt_jump(uint32_t seed, uint64_t n, uint32_t* out, int num_sms, int log_seg, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const mt::Tables& T = mt::tables();
    if (!T.ok) return cudaErrorInvalidValue;
    const uint64_t* dj = nullptr;
    cudaError_t e = mt::device_table(T, &dj);
    if (e != cudaSuccess) return e;
    const int logS = log_seg > 0 ? log_seg : choose_log_seg(n, num_sms);
    if (logS < 10) return cudaErrorInvalidValue;  // a segment holds at least its window
    const uint64_t nseg = (n + (1ull << logS) - 1) >> logS;
    int top = 0;
    while ((nseg - 1) >> top) ++top;
    if (logS + top > mt::MAXB || nseg > 0x7fffffffull) return cudaErrorInvalidValue;
    const size_t smem = mt_jump_smem();
    if ((e = cudaFuncSetAttribute(mt::k_mt_windows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
        cudaSuccess)
        return e;
    mt::k_mt_windows<<<(unsigned)nseg, mt::WTHREADS, smem, s>>>(seed, n, logS, dj, out);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    mt::k_mt_generate<<<(unsigned)nseg, mt::GTHREADS, 0, s>>>(n, logS, out);
    return cudaGetLastError();
}

void mt_release_device_tables() {
    std::lock_guard<std::mutex> lk(mt::g_mu);
    for (mt::DeviceTable& d : mt::g_dev) cudaFree(d.p);
    mt::g_dev.clear();
}

int mt_window_host(uint32_t seed, uint64_t offset, uint32_t* window) {
    const mt::Tables& T = mt::tables();
    if (!T.ok) return -1;
    mt::first_window(seed, window);
    for (int b = 0; b < mt::MAXB && (offset >> b); ++b)
        if ((offset >> b) & 1ull) mt::apply_host(window, T.jump.data() + (size_t)b * mt::PW);
    return (offset >> mt::MAXB) ? -1 : 0;
}

}  // namespace rrsw
