// k_lj92.cu -- the DNG lossless-JPEG decoder (DecodeLosslessJPEG, src/gls_dng_lossless_jpeg.cpp,
// called per tile or strip by the DNG reader, src/gls_image_tiff.cpp:369-440) on the GPU.
//
// A lossless-JPEG scan is a Huffman-coded sequence of MCUs (one difference per component);
// the samples are the running sums of the differences along the predictor.  The reference
// decodes it serially.  Here:
//   1. the host parses each stream's marker segments (tables, frame, scan, restart
//      interval) exactly as the reference does, and one copy brings the data to the device;
//   2. de-stuffing on the device: each restart interval's entropy-coded bytes end at the
//      first FF not followed by 00; the 00 after every data FF is dropped (chunked counts,
//      per-interval offsets, compaction);
//   3. speculative decoding: the de-stuffed bits of an interval are cut into segments of
//      kSegBits; a thread decodes units (single codewords when all the scan's tables split
//      bits alike, else whole MCUs) from the start of its segment to the first unit
//      boundary past its end.  A decode unit of one codeword has no component phase to
//      lose: a decode started on the wrong component of a multi-component scan stays in
//      step once its bits are.  Huffman codes resynchronise, so a thread started at a wrong
//      bit soon falls onto the true unit boundaries; kSyncRounds parallel rounds re-decode a
//      segment from the end its predecessor reached, then one thread per interval walks the
//      segments still out of step (exact, serial only where the rounds left work).  A scan
//      of the per-segment unit counts gives every segment its first unit index, and a last
//      pass decodes again and writes the differences;
//   4. reconstruction: column 0 runs down the rows (predictor: the row above, the
//      interval's first row starting from 2^(P-Pt-1)); predictor 1 rows are prefix sums
//      (one block per row); the other predictors go row after row, in parallel over the
//      columns where the predictor does not use the left neighbour;
//   5. the samples of each stream are laid out as its tile (tile_width per row), clipped
//      at the image border, as the reference's tile loop does.
// The Huffman decode is the reference's own procedure (8-bit lookup, then the canonical
// walk; an invalid code consumes 17 bits and decodes as category 0; category 16 is -32768
// without extra bits), and past the end of an interval's data the bits read as zeros.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gls_internal.h"

namespace gls {
namespace {

constexpr int kSegBits = 2048;    // bits per speculative segment
constexpr int kChunk = 4096;      // source bytes per de-stuffing chunk
constexpr int kSyncRounds = 2;    // parallel resynchronisation rounds before the walk
constexpr int kPad = 16;          // zero bytes after each interval's de-stuffed data
constexpr int kBnd = 8;           // unit starts remembered per segment from the first pass

struct LjTable {
    uint16_t look[256];  // (code length << 8) | value for codes of at most 8 bits; 0: longer
    int maxcode[18];
    int mincode[17];
    int valptr[17];
    uint8_t val[256];
};

struct LjStream {
    int width, height, comps, precision, predictor, pt;
    // codewords per decode unit: comps (one MCU), or 1 when every table of the scan splits
    // bits into codewords alike (then where a codeword starts does not depend on its
    // component, which the codeword's index gives)
    int upc;
    int zero_unit_bits;  // bits of a unit of all-zero codewords decoding to 0 differences (0: none)
    int table[4];
    long long sample_off;  // first sample of the stream in the samples buffer
    int tile_x, tile_y, clip_w, clip_h;  // placement of the stream's samples in the image
    int tile_w;                          // samples per tile row
    int interval_base, nint;
    int row_base;  // first global row of the stream
};

struct LjInterval {
    long long src_begin, src_limit;  // entropy-coded bytes (device offsets)
    long long dst_off;               // de-stuffed bytes (4-byte aligned, kPad zero bytes after)
    long long dst_words;             // 32-bit words the interval owns in the de-stuffed buffer
    long long mcu_off;               // first MCU of the interval within its stream
    int stream, first_row, rows;
    int seg_base, nseg, chunk_base, nchunk;
};

struct LjChunk {
    long long begin, end;
    int interval;
};

struct LjDev {
    const uint8_t* src;
    uint8_t* dst;
    const LjStream* streams;
    const LjInterval* intervals;
    const LjChunk* chunks;
    const LjTable* tables;
    const int* seg_interval;
    const int* row_stream;
    unsigned long long* marker;  // per interval: first marker position (init src_limit)
    long long* dlen;             // per interval: de-stuffed bytes
    int* chunk_stuff;
    long long* chunk_off;
    long long* start_used;  // per segment
    long long* bnd;         // per segment: the first kBnd MCU starts of the pass-1 decode
    int* p1cnt;             // per segment: units of the pass-1 decode (from the segment's first bit)
    int8_t* p1;             // per segment: the segment's values are still the pass-1 decode
    long long* end_a;
    long long* end_b;
    int* cnt;
    long long* seg_off;
    int* error;
    int16_t* diff;
    uint16_t* recon;
    uint16_t* out;
    int out_pitch;
};

__device__ __forceinline__ uint32_t bswap32(uint32_t v) { return __byte_perm(v, 0, 0x0123); }

// 32 bits of an interval's de-stuffed data from bit pos; words past the interval read as 0
struct BitSrc {
    const uint32_t* w;
    long long nwords;
};

__device__ __forceinline__ uint32_t peek32(const BitSrc& b, long long pos) {
    const long long i = pos >> 5;
    const uint32_t hi = i < b.nwords ? bswap32(__ldg(b.w + i)) : 0u;
    const uint32_t lo = i + 1 < b.nwords ? bswap32(__ldg(b.w + i + 1)) : 0u;
    const uint64_t v = ((uint64_t)hi << 32) | lo;
    return (uint32_t)(v << (pos & 31) >> 32);
}

__device__ __forceinline__ BitSrc bits_of(const uint8_t* dst, const LjInterval& iv) {
    return BitSrc{reinterpret_cast<const uint32_t*>(dst + iv.dst_off), iv.dst_words};
}

// Length of the run of zero bits at pos, at most cap.
__device__ __forceinline__ long long zero_run(const BitSrc& b, long long pos, long long cap) {
    long long r = 0;
    const uint32_t v = peek32(b, pos);
    if (v) return min(cap, (long long)__clz(v));
    r = 32 - (pos & 31);  // to the next word boundary
    long long w = (pos >> 5) + 1;
    while (r < cap) {
        const uint32_t x = w < b.nwords ? bswap32(__ldg(b.w + w)) : 0u;
        if (x) return min(cap, r + __clz(x));
        r += 32;
        w++;
    }
    return cap;
}

// Units of all-zero codewords that fit wholly in the zero run at pos (at most max_units): a
// flat area of the image is such a run, and its units all decode to zero differences.
__device__ __forceinline__ long long zero_units(const LjStream& st, const BitSrc& b, long long pos,
                                                long long max_units) {
    if (st.zero_unit_bits == 0 || max_units <= 0 || peek32(b, pos) != 0) return 0;
    const long long P = st.zero_unit_bits;
    return min(max_units, zero_run(b, pos, max_units * P) / P);
}

// Sequential reader over an interval's de-stuffed bits: a 64-bit buffer of the next bits
// (most significant first, at least 33 valid after every step) and the word after them
// loaded ahead, so a serial decode waits on a memory load only once per 32 bits consumed.
struct BitReader {
    const uint32_t* w;
    long long nwords;
    long long widx;  // index of the word held in nw
    long long pos;   // bit position of the buffer's first bit
    uint64_t acc;
    int avail;
    uint32_t nw;
    __device__ __forceinline__ uint32_t word(long long i) const { return i < nwords ? bswap32(__ldg(w + i)) : 0u; }
    __device__ __forceinline__ void refill() {
        if (avail <= 32) {
            acc |= (uint64_t)nw << (32 - avail);
            avail += 32;
            widx++;
            nw = word(widx);
        }
    }
    __device__ __forceinline__ void seek(long long p) {
        pos = p;
        const long long i = p >> 5;
        const int o = (int)(p & 31);
        acc = (uint64_t)word(i) << (32 + o);
        avail = 32 - o;
        widx = i + 1;
        nw = word(widx);
        refill();
    }
    __device__ __forceinline__ uint32_t peek() const { return (uint32_t)(acc >> 32); }
    __device__ __forceinline__ void skip(int n) {  // n <= 32
        acc <<= n;
        avail -= n;
        pos += n;
        refill();
    }
};

__device__ __forceinline__ BitReader reader_at(const BitSrc& b, long long pos) {
    BitReader r;
    r.w = b.w;
    r.nwords = b.nwords;
    r.seek(pos);
    return r;
}

// One difference: HuffDecode + HuffExtend (gls_dng_lossless_jpeg.cpp:1424-1500), on the
// reader (a code of at most 16 bits and at most 15 extra bits, or an invalid code of 17
// bits: never more than 32 bits at a time).  Returns the bits consumed; *bad is set for a
// category above 16 (the reference throws).
__device__ __forceinline__ int decode_diff_r(const LjTable* __restrict__ t, BitReader& br, int* d, bool* bad) {
    const uint32_t v = br.peek();
    const uint32_t c8 = v >> 24;
    const uint32_t lk = t->look[c8];
    int len, s;
    if (lk) {
        len = (int)(lk >> 8);
        s = (int)(lk & 0xFF);
    } else {
        int code = (int)c8, l = 8;
        while (code > t->maxcode[l]) {
            code = (code << 1) | (int)((v >> (31 - l)) & 1u);
            l++;
        }
        len = l;
        if (l > 16) {
            s = 0;
        } else {
            int idx = t->valptr[l] + (code - t->mincode[l]);
            idx = idx < 0 ? 0 : (idx > 255 ? 255 : idx);
            s = t->val[idx];
        }
    }
    if (s == 0) {
        *d = 0;
    } else if (s == 16) {
        *d = -32768;
    } else if (s > 16) {
        *bad = true;
        *d = 0;
    } else {
        int x = (int)((v << len) >> (32 - s));
        if (x < (0x8000 >> (16 - s))) x += (-1 << s) + 1;
        *d = x;
        len += s;
    }
    br.skip(len);
    return len;
}

// One decode unit whose first codeword belongs to component comp0 (always 0 for a whole
// MCU; a single codeword may sit at any component).
__device__ __forceinline__ int unit_bits_r(const LjDev& g, const LjStream& st, BitReader& br, int comp0, int* d,
                                           bool* bad) {
    int used = 0;
    for (int k = 0; k < st.upc; k++) {
        const int c = comp0 + k < st.comps ? comp0 + k : comp0 + k - st.comps;
        used += decode_diff_r(g.tables + st.table[c], br, d + k, bad);
    }
    return used;
}

// ---- de-stuffing ----

__global__ void lj_marker_kernel(LjDev g) {
    const LjChunk c = g.chunks[blockIdx.x];
    const LjInterval iv = g.intervals[c.interval];
    unsigned long long best = ~0ull;
    for (long long i = c.begin + threadIdx.x; i < c.end; i += blockDim.x) {
        if (g.src[i] == 0xFF) {
            const int next = i + 1 < iv.src_limit ? g.src[i + 1] : 0xFF;
            if (next != 0) best = min(best, (unsigned long long)i);
        }
    }
    for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0 && best != ~0ull) atomicMin(&g.marker[c.interval], best);
}

__global__ void lj_stuff_count_kernel(LjDev g) {
    const LjChunk c = g.chunks[blockIdx.x];
    const LjInterval iv = g.intervals[c.interval];
    const long long end = min(c.end, (long long)g.marker[c.interval]);
    int n = 0;
    for (long long i = c.begin + threadIdx.x; i < end; i += blockDim.x)
        n += (i > iv.src_begin && g.src[i - 1] == 0xFF);
    for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
    __shared__ int s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = n;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s[w];
        g.chunk_stuff[blockIdx.x] = t;
    }
}

// Block-wide exclusive scan of one value per thread (blockDim.x = 256) with a running
// carry across calls; returns the thread's exclusive prefix and adds the block total to
// *carry (shared).
template <class T>
__device__ __forceinline__ T block_exclusive(T v, T* carry) {
    __shared__ T s_w[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    T incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const T t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    T base = *carry + incl - v, tot = 0;
    for (int w = 0; w < 8; w++) {
        if (w < warp) base += s_w[w];
        tot += s_w[w];
    }
    __syncthreads();
    if (threadIdx.x == 0) *carry += tot;
    __syncthreads();
    return base;
}

// one block per interval: chunk output offsets and the de-stuffed length
__global__ void __launch_bounds__(256) lj_chunk_offsets_kernel(LjDev g) {
    const LjInterval iv = g.intervals[blockIdx.x];
    const long long m = (long long)g.marker[blockIdx.x];
    __shared__ long long s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int b = 0; b < iv.nchunk; b += 256) {
        const int c = iv.chunk_base + b + threadIdx.x;
        long long kept = 0;
        if (b + (int)threadIdx.x < iv.nchunk) {
            const LjChunk ch = g.chunks[c];
            kept = max(0ll, min(ch.end, m) - ch.begin) - g.chunk_stuff[c];
        }
        const long long off = block_exclusive<long long>(kept, &s_carry);
        if (b + (int)threadIdx.x < iv.nchunk) g.chunk_off[c] = off;
    }
    if (threadIdx.x == 0) g.dlen[blockIdx.x] = s_carry;
}

__global__ void __launch_bounds__(256) lj_destuff_kernel(LjDev g) {
    constexpr int kPer = kChunk / 256;
    const LjChunk c = g.chunks[blockIdx.x];
    const LjInterval iv = g.intervals[c.interval];
    const long long end = min(c.end, (long long)g.marker[c.interval]);
    const long long b0 = c.begin + (long long)threadIdx.x * kPer;
    uint8_t v[kPer];
    int keep = 0;
    unsigned mask = 0;
#pragma unroll
    for (int j = 0; j < kPer; j++) {
        const long long i = b0 + j;
        v[j] = 0;
        if (i < end && !(i > iv.src_begin && g.src[i - 1] == 0xFF)) {
            v[j] = g.src[i];
            mask |= 1u << j;
            keep++;
        }
    }
    // block exclusive scan of keep
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = keep;
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    __shared__ int s_w[8];
    if (lane == 31) s_w[warp] = incl;
    __syncthreads();
    int base = incl - keep;
    for (int w = 0; w < warp; w++) base += s_w[w];
    uint8_t* out = g.dst + iv.dst_off + g.chunk_off[blockIdx.x] + base;
    int k = 0;
#pragma unroll
    for (int j = 0; j < kPer; j++)
        if (mask & (1u << j)) out[k++] = v[j];
}

// ---- speculative decoding ----

__device__ __forceinline__ void seg_decode(const LjDev& g, int seg, long long start, long long* end_out,
                                           int* cnt_out, long long* bnd = nullptr) {
    const int I = g.seg_interval[seg];
    const LjInterval iv = g.intervals[I];
    const LjStream st = g.streams[iv.stream];
    const BitSrc base = bits_of(g.dst, iv);
    const int j = seg - iv.seg_base;
    const long long limit = (long long)(j + 1) * kSegBits;
    const long long total = (long long)iv.rows * st.width * st.comps / st.upc;
    BitReader br = reader_at(base, start);
    int n = 0;
    bool bad = false;
    int d[4];
    while (br.pos < limit && (j > 0 || n < total)) {
        if (st.zero_unit_bits && br.peek() == 0) {
            const long long pos = br.pos;
            const long long want = (limit - pos + st.zero_unit_bits - 1) / st.zero_unit_bits;
            const long long z = zero_units(st, base, pos, j > 0 ? want : min(want, total - n));
            if (z > 0) {
                if (bnd)
                    for (long long m = 0; m < z && n + m < kBnd; m++) bnd[n + m] = pos + m * st.zero_unit_bits;
                br.seek(pos + z * st.zero_unit_bits);
                n += (int)z;
                continue;
            }
        }
        if (bnd && n < kBnd) bnd[n] = br.pos;
        unit_bits_r(g, st, br, 0, d, &bad);  // positions only: any component parses alike
        n++;
    }
    if (bnd)
        for (int k = n; k < kBnd; k++) bnd[k] = -1;
    *end_out = br.pos;
    *cnt_out = n;
}

__global__ void lj_phase1_kernel(LjDev g, int nseg) {
    const int seg = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg >= nseg) return;
    const int I = g.seg_interval[seg];
    const LjInterval iv = g.intervals[I];
    const int j = seg - iv.seg_base;
    const long long start = (long long)j * kSegBits;
    g.start_used[seg] = start;
    if (j > 0 && start >= g.dlen[I] * 8) {
        g.end_a[seg] = start;
        g.cnt[seg] = 0;
        g.p1[seg] = 0;
        return;
    }
    long long e;
    int n;
    seg_decode(g, seg, start, &e, &n, g.bnd + (size_t)seg * kBnd);
    g.end_a[seg] = e;
    g.cnt[seg] = n;
    g.p1cnt[seg] = n;
    g.p1[seg] = 1;
}

// One resynchronisation round: a segment whose start differs from the end its predecessor
// reached re-decodes from there.  Reads end_in, writes end_out (double-buffered).
__global__ void lj_sync_kernel(LjDev g, int nseg, const long long* end_in, long long* end_out) {
    const int seg = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg >= nseg) return;
    const int I = g.seg_interval[seg];
    const LjInterval iv = g.intervals[I];
    const int j = seg - iv.seg_base;
    const long long mine = end_in[seg];
    end_out[seg] = mine;
    // the first segment starts on a true boundary; segments past the data stay empty
    if (j == 0 || (long long)j * kSegBits >= g.dlen[I] * 8) return;
    const long long s = end_in[seg - 1];
    if (s == g.start_used[seg]) return;
    if (g.p1[seg]) {  // the new start is a unit start of the first pass: the rest of its path
        const long long* b = g.bnd + (size_t)seg * kBnd;
        for (int k = 0; k < kBnd; k++)
            if (b[k] == s) {
                g.start_used[seg] = s;
                g.cnt[seg] = g.p1cnt[seg] - k;
                return;
            }
    }
    long long e;
    int n;
    seg_decode(g, seg, s, &e, &n);
    g.start_used[seg] = s;
    g.cnt[seg] = n;
    g.p1[seg] = 0;
    end_out[seg] = e;
}

// Parallel repair: one thread per maximal run of consecutive segments whose start is not
// their predecessor's end; it re-decodes the run from the end before it and stops at the
// end of the run once the end no longer moves.  A thread writes only its own run, so
// threads never share a segment; what is left out of step (a run whose end still moves,
// a run that started from an end another thread changed) is the serial walk's.
__global__ void lj_repair_kernel(LjDev g, int nseg, const long long* ends_in, long long* ends_out) {
    const int seg = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg >= nseg) return;
    const int I = g.seg_interval[seg];
    const LjInterval iv = g.intervals[I];
    const int j = seg - iv.seg_base;
    const long long nbits = g.dlen[I] * 8;
    // out of step on entry (reads only values no thread writes before it is decided)
    auto out_of_step = [&](int k) {
        return k > 0 && k < iv.nseg && (long long)k * kSegBits < nbits &&
               g.start_used[iv.seg_base + k] != ends_in[iv.seg_base + k - 1];
    };
    const bool mine = out_of_step(j);
    if (!mine) {
        ends_out[seg] = ends_in[seg];
        return;
    }
    if (out_of_step(j - 1)) return;  // inside a run: its first segment's thread handles it
    int k = j;
    long long start = ends_in[seg - 1];
    for (;;) {
        const int sk = iv.seg_base + k;
        const bool next = out_of_step(k + 1);
        long long e;
        int n;
        seg_decode(g, sk, start, &e, &n);
        g.start_used[sk] = start;
        g.cnt[sk] = n;
        g.p1[sk] = 0;
        ends_out[sk] = e;
        if (!next) break;
        k++;
        start = e;
    }
}

// After the parallel rounds, per interval: the segments whose start is not the end of
// their predecessor are listed (in order) and one thread walks the list, re-decoding each
// from its predecessor's end and carrying on into the following segments while the end
// moves.  Exact whatever the rounds left behind; the serial work is only what they did not
// resolve (a periodic stretch of the bitstream, e.g. a flat area, can keep a speculative
// decode on the wrong component for many segments).
__global__ void __launch_bounds__(256) lj_walk_kernel(LjDev g, long long* ends, int* list) {
    const int I = blockIdx.x;
    const LjInterval iv = g.intervals[I];
    const long long nbits = g.dlen[I] * 8;
    const int nact = (int)min((long long)iv.nseg, max(1ll, (nbits + kSegBits - 1) / kSegBits));
    __shared__ int s_n;
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    for (int b = 1; b < nact; b += 256 * 16) {
        const int j0 = b + threadIdx.x * 16;
        unsigned f = 0;
#pragma unroll
        for (int k = 0; k < 16; k++) {
            const int j = j0 + k;
            if (j < nact && g.start_used[iv.seg_base + j] != ends[iv.seg_base + j - 1]) f |= 1u << k;
        }
        int off = block_exclusive<int>(__popc(f), &s_n);
        for (int k = 0; k < 16; k++)
            if (f & (1u << k)) list[iv.seg_base + off++] = j0 + k;
    }
    if (threadIdx.x != 0) return;
    int fixed = 0;
    for (int q = 0; q < s_n; q++) {
        int k = list[iv.seg_base + q];
        if (k <= fixed) continue;
        long long start = ends[iv.seg_base + k - 1];
        for (;;) {
            const int seg = iv.seg_base + k;
            long long e;
            int n;
            seg_decode(g, seg, start, &e, &n);
            const long long old = ends[seg];
            g.start_used[seg] = start;
            g.cnt[seg] = n;
            g.p1[seg] = 0;
            ends[seg] = e;
            fixed = k;
            if (e == old || k + 1 >= nact) break;
            k++;
            start = e;
        }
    }
}

constexpr int kScanPer = 16;  // consecutive elements per thread in the per-interval scans

// per interval: exclusive scan of the segment counts (one block per interval, kScanPer
// consecutive segments per thread)
__global__ void __launch_bounds__(256) lj_count_scan_kernel(LjDev g) {
    const LjInterval iv = g.intervals[blockIdx.x];
    __shared__ long long s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int b = 0; b < iv.nseg; b += 256 * kScanPer) {
        const int j0 = b + threadIdx.x * kScanPer;
        long long v[kScanPer], tot = 0;
#pragma unroll
        for (int k = 0; k < kScanPer; k++) {
            v[k] = j0 + k < iv.nseg ? g.cnt[iv.seg_base + j0 + k] : 0;
            tot += v[k];
        }
        long long off = block_exclusive<long long>(tot, &s_carry);
#pragma unroll
        for (int k = 0; k < kScanPer; k++) {
            if (j0 + k < iv.nseg) g.seg_off[iv.seg_base + j0 + k] = off;
            off += v[k];
        }
    }
}

__global__ void lj_write_kernel(LjDev g, int nseg) {
    const int seg = blockIdx.x * blockDim.x + threadIdx.x;
    if (seg >= nseg) return;
    const int I = g.seg_interval[seg];
    const LjInterval iv = g.intervals[I];
    const LjStream st = g.streams[iv.stream];
    const int j = seg - iv.seg_base;
    const long long nbits = g.dlen[I] * 8;
    if (j > 0 && (long long)j * kSegBits >= nbits) return;  // past the data
    // the segment holding the end of the data decodes on until the interval is complete
    const bool last = (long long)(j + 1) * kSegBits >= nbits;
    const long long limit = (long long)(j + 1) * kSegBits;
    const int U = st.upc;
    const long long total = (long long)iv.rows * st.width * st.comps / U;
    const BitSrc base = bits_of(g.dst, iv);
    BitReader br = reader_at(base, g.start_used[seg]);
    long long m = g.seg_off[seg];
    int16_t* out = g.diff + st.sample_off + iv.mcu_off * st.comps;
    bool bad = false;
    int d[4];
    while (m < total && (br.pos < limit || last)) {
        if (st.zero_unit_bits && br.peek() == 0) {
            const long long pos = br.pos;
            const long long want =
                last ? total - m : min(total - m, (limit - pos + st.zero_unit_bits - 1) / st.zero_unit_bits);
            const long long z = zero_units(st, base, pos, want);
            if (z > 0) {
                for (long long q = m * U; q < (m + z) * U; q++) out[q] = 0;
                br.seek(pos + z * st.zero_unit_bits);
                m += z;
                continue;
            }
        }
        // the interval starts on an MCU, so codeword m * U belongs to component (m * U) % comps
        unit_bits_r(g, st, br, (int)((m * U) % st.comps), d, &bad);
        for (int k = 0; k < U; k++) out[m * U + k] = (int16_t)d[k];
        m++;
    }
    if (bad) atomicExch(g.error, 1);
}

// ---- reconstruction ----

// column 0 of every row: one block per (interval, component), a prefix sum down the rows
// from 2^(P-Pt-1)
__global__ void __launch_bounds__(256) lj_col0_kernel(LjDev g) {
    const int I = blockIdx.x >> 2, k = blockIdx.x & 3;
    const LjInterval iv = g.intervals[I];
    const LjStream st = g.streams[iv.stream];
    if (k >= st.comps) return;
    const long long rowlen = (long long)st.width * st.comps;
    const long long base = st.sample_off + (long long)iv.first_row * rowlen + k;
    __shared__ uint32_t s_carry;
    if (threadIdx.x == 0) s_carry = 1u << (st.precision - st.pt - 1);
    __syncthreads();
    for (int b = 0; b < iv.rows; b += 256) {
        const int r = b + threadIdx.x;
        const uint32_t d = r < iv.rows ? (uint32_t)(int)g.diff[base + r * rowlen] : 0u;
        const uint32_t x = block_exclusive<uint32_t>(d, &s_carry) + d;
        if (r < iv.rows) g.recon[base + r * rowlen] = (uint16_t)x;
    }
}

// rows predicted from the left (predictor 1 everywhere, and every interval's first row):
// one block per row, prefix sums of the differences per component
__global__ void __launch_bounds__(256) lj_row_scan_kernel(LjDev g, int nrows) {
    const int gr = blockIdx.x;
    if (gr >= nrows) return;
    const int s = g.row_stream[gr];
    const LjStream st = g.streams[s];
    const int r = gr - st.row_base;
    bool first = r == 0;
    if (!first && st.nint > 1) {  // first row of its restart interval?
        const int per = g.intervals[st.interval_base].rows;
        first = per > 0 && r % per == 0;
    }
    if (st.predictor != 1 && !first) return;
    const int C = st.comps;
    const long long rowbase = st.sample_off + (long long)r * st.width * C;
    const int n = st.width - 1;  // MCUs after column 0
    const int per_thread = (n + blockDim.x - 1) / blockDim.x;
    const int m0 = 1 + threadIdx.x * per_thread;
    const int m1 = min(st.width, m0 + per_thread);
    uint32_t sum[4] = {0, 0, 0, 0};
    for (int m = m0; m < m1; m++)
        for (int k = 0; k < C; k++) sum[k] += (uint32_t)(int)g.diff[rowbase + (long long)m * C + k];
    // block exclusive scan of sum[0..C)
    __shared__ uint32_t s_w[8][4];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t excl[4];
    for (int k = 0; k < 4; k++) {
        uint32_t incl = sum[k];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) s_w[warp][k] = incl;
        excl[k] = incl - sum[k];
    }
    __syncthreads();
    for (int k = 0; k < C; k++) {
        uint32_t x = excl[k] + (uint32_t)g.recon[rowbase + k];
        for (int w = 0; w < warp; w++) x += s_w[w][k];
        for (int m = m0; m < m1; m++) {
            const long long i = rowbase + (long long)m * C + k;
            x += (uint32_t)(int)g.diff[i];
            g.recon[i] = (uint16_t)x;
        }
    }
}

__device__ __forceinline__ int lj_predict(int ss, int left, int upper, int diag) {
    switch (ss) {
        case 0: return 0;
        case 1: return left;
        case 2: return upper;
        case 3: return diag;
        case 4: return left + upper - diag;
        case 5: return left + ((upper - diag) >> 1);
        case 6: return upper + ((left - diag) >> 1);
        default: return (left + upper) >> 1;
    }
}

// predictors other than 1, rows after the first of each interval: one block per interval,
// row after row (QuickPredict, gls_dng_lossless_jpeg.cpp:1258-1296)
__global__ void __launch_bounds__(256) lj_rows_general_kernel(LjDev g, int nint) {
    const LjInterval iv = g.intervals[blockIdx.x];
    const LjStream st = g.streams[iv.stream];
    if (st.predictor == 1) return;
    const int C = st.comps;
    const long long rowlen = (long long)st.width * C;
    for (int r = 1; r < iv.rows; r++) {
        const long long row = st.sample_off + (long long)(iv.first_row + r) * rowlen;
        const long long prev = row - rowlen;
        if (st.predictor == 0 || st.predictor == 2 || st.predictor == 3) {
            for (long long i = C + threadIdx.x; i < rowlen; i += blockDim.x) {
                const int p = lj_predict(st.predictor, 0, g.recon[prev + i], g.recon[prev + i - C]);
                g.recon[row + i] = (uint16_t)((int)g.diff[row + i] + p);
            }
        } else if (threadIdx.x < C) {
            const int k = threadIdx.x;
            int left = g.recon[row + k];
            for (int m = 1; m < st.width; m++) {
                const long long i = (long long)m * C + k;
                const int p = lj_predict(st.predictor, left, g.recon[prev + i], g.recon[prev + i - C]);
                left = (uint16_t)((int)g.diff[row + i] + p);
                g.recon[row + i] = (uint16_t)left;
            }
        }
        __syncthreads();
    }
}

// samples -> image: one block per stream row
__global__ void lj_place_kernel(LjDev g, int nrows) {
    const int gr = blockIdx.x;
    if (gr >= nrows) return;
    const LjStream st = g.streams[g.row_stream[gr]];
    const int r = gr - st.row_base;
    const long long rowlen = (long long)st.width * st.comps;
    const long long q0 = (long long)r * rowlen;
    for (long long i = threadIdx.x; i < rowlen; i += blockDim.x) {
        const long long q = q0 + i;
        const int ty = (int)(q / st.tile_w), tx = (int)(q - (long long)ty * st.tile_w);
        if (tx < st.clip_w && ty < st.clip_h)
            g.out[(size_t)(st.tile_y + ty) * g.out_pitch + st.tile_x + tx] = g.recon[st.sample_off + q];
    }
}

// ---- host: marker segments (ReadFileHeader / ReadScanHeader, gls_dng_lossless_jpeg.cpp:540-1075) ----

struct HostTable {
    uint8_t bits[17] = {};
    uint8_t val[256] = {};
    bool present = false;
};

struct HostHeader {
    int precision = 0, width = 0, height = 0, ncomp = 0, ns = 0, ss = 0, pt = 0, restart = 0;
    int scan_table[4] = {};
    size_t scan_pos = 0;
    HostTable tab[4];
};

struct ByteReader {
    const uint8_t* d;
    size_t n, pos;
    bool ok = true;
    int get() {
        if (pos >= n) {
            ok = false;
            return 0;
        }
        return d[pos++];
    }
    int get2() {
        const int a = get();
        return (a << 8) | get();
    }
    int marker() {
        int c;
        do {
            do c = get(); while (ok && c != 0xFF);
            do c = get(); while (ok && c == 0xFF);
        } while (ok && c == 0);
        return ok ? c : -1;
    }
};

int process_tables(ByteReader& b, HostHeader& h) {
    for (;;) {
        const int c = b.marker();
        if (c < 0) return -1;
        if ((c >= 0xC0 && c <= 0xCF && c != 0xC4 && c != 0xCC) || c == 0xD8 || c == 0xD9 || c == 0xDA) return c;
        if (c == 0xC4) {
            int len = b.get2() - 2;
            while (len > 0 && b.ok) {
                const int idx = b.get();
                if (idx >= 4) return -1;
                HostTable& t = h.tab[idx];
                t.present = true;
                int count = 0;
                for (int i = 1; i <= 16; i++) count += (t.bits[i] = (uint8_t)b.get());
                if (count > 256) return -1;
                for (int j = 0; j < count; j++) t.val[j] = (uint8_t)b.get();
                len -= 1 + 16 + count;
            }
        } else if (c == 0xDB || (c >= 0xD0 && c <= 0xD7) || c == 0x01) {
        } else if (c == 0xDD) {
            if (b.get2() != 4) return -1;
            h.restart = b.get2();
        } else {
            const size_t len = (size_t)(b.get2() - 2);
            if (b.pos + len >= b.n) return -1;
            b.pos += len;
        }
        if (!b.ok) return -1;
    }
}

bool parse_header(const uint8_t* d, size_t n, HostHeader& h) {
    ByteReader b{d, n, 0};
    if (b.get() != 0xFF || b.get() != 0xD8) return false;
    int c = process_tables(b, h);
    if (c != 0xC0 && c != 0xC1 && c != 0xC3) return false;
    const int len = b.get2();
    h.precision = b.get();
    h.height = b.get2();
    h.width = b.get2();
    h.ncomp = b.get();
    if (h.height <= 0 || h.width <= 0 || h.ncomp <= 0 || h.precision < 2 || h.precision > 16) return false;
    if (len != h.ncomp * 3 + 8) return false;
    int ids[256];
    for (int i = 0; i < h.ncomp; i++) {
        ids[i] = b.get();
        const int hv = b.get();
        b.get();
        if (hv != 0x11) return false;  // DecoderStructInit: 1x1 sampling only
    }
    c = process_tables(b, h);
    if (c != 0xDA) return false;
    const int slen = b.get2() - 3;
    h.ns = b.get();
    if (slen != h.ns * 2 + 3 || h.ns < 1 || h.ns > 4) return false;
    for (int i = 0; i < h.ns; i++) {
        const int cc = b.get(), tt = b.get();
        int ci = 0;
        while (ci < h.ncomp && ids[ci] != cc) ci++;
        if (ci >= h.ncomp) return false;
        h.scan_table[i] = (tt >> 4) & 15;
        if (h.scan_table[i] > 3 || !h.tab[h.scan_table[i]].present) return false;
    }
    h.ss = b.get();
    b.get();
    h.pt = b.get() & 0x0F;
    if (h.pt >= h.precision) return false;
    h.scan_pos = b.pos;
    return b.ok;
}

// FixHuffTbl (gls_dng_lossless_jpeg.cpp:200-316): canonical codes, bounds, 8-bit lookup
void derive_table(const HostTable& h, LjTable& t) {
    int size[257], code[257], n = 0;
    for (int l = 1; l <= 16; l++)
        for (int i = 0; i < h.bits[l]; i++) size[n++] = l;
    size[n] = 0;
    int c = 0, si = size[0], p = 0;
    while (size[p]) {
        while (size[p] == si) code[p++] = c++;
        c <<= 1;
        si++;
    }
    memset(&t, 0, sizeof(t));
    memcpy(t.val, h.val, 256);
    p = 0;
    for (int l = 1; l <= 16; l++) {
        if (h.bits[l]) {
            t.valptr[l] = p;
            t.mincode[l] = code[p] & 0xFFFF;
            p += h.bits[l];
            t.maxcode[l] = code[p - 1];
        } else {
            t.maxcode[l] = -1;
        }
    }
    t.maxcode[17] = 0xFFFFF;
    for (int q = 0; q < n; q++)
        if (size[q] <= 8) {
            const int lo = code[q] << (8 - size[q]), hi = size[q] < 8 ? lo | ((1 << (8 - size[q])) - 1) : lo;
            for (int k = lo; k <= hi && k < 256; k++) t.look[k] = (uint16_t)((size[q] << 8) | h.val[q]);
        }
}

// Whether two tables split every bit string into codewords of the same lengths: the same
// number of codes of each length (so the same canonical codes) and, code by code, the same
// number of extra bits (category s < 16 reads s bits, 16 none; a category above 16 is an
// error and must match exactly).
bool same_parse(const HostTable& a, const HostTable& b) {
    int n = 0;
    for (int l = 1; l <= 16; l++) {
        if (a.bits[l] != b.bits[l]) return false;
        n += a.bits[l];
    }
    auto extra = [](int s) { return s < 16 ? s : (s == 16 ? 0 : -s); };
    for (int p = 0; p < n && p < 256; p++)
        if (extra(a.val[p]) != extra(b.val[p])) return false;
    return true;
}

template <class T>
size_t carve(size_t& off, size_t count) {
    const size_t o = (off + 255) & ~(size_t)255;
    off = o + count * sizeof(T);
    return o;
}

}  // namespace
}  // namespace gls

using namespace gls;

extern "C" gls_status gls_lossless_jpeg_info(const uint8_t* data, size_t size, gls_ljpeg_info* info) {
    if (!data || !info) return GLS_ERR_INVALID_ARGUMENT;
    HostHeader h;
    if (size < 4 || !parse_header(data, size, h)) return GLS_ERR_BAD_STREAM;
    // the decoder's predictor rule (QuickPredict, gls_dng_lossless_jpeg.cpp:1290)
    if (h.ss > 7 && h.width > 1 && h.height > 1 && h.restart / h.width != 1) return GLS_ERR_BAD_STREAM;
    bool alike = true;
    for (int k = 1; k < h.ns; k++) alike = alike && same_parse(h.tab[h.scan_table[0]], h.tab[h.scan_table[k]]);
    info->width = h.width;
    info->height = h.height;
    info->components = h.ns;
    info->precision = h.precision;
    info->predictor = h.ss;
    info->point_transform = h.pt;
    info->restart_interval = h.restart;
    info->tables_alike = alike ? 1 : 0;
    return GLS_OK;
}

extern "C" gls_status gls_dng_decode_lossless_jpeg(gls_ctx* ctx, const uint8_t* data, size_t data_size, int n_streams,
                                                   const uint64_t* offsets, const uint64_t* sizes, int tile_width,
                                                   int tile_height, const gls_image_desc* out) {
    if (!ctx) return GLS_ERR_INVALID_ARGUMENT;
    GLS_CHECK(check_desc(ctx, out, "out", GLS_R16_UNORM));
    if (!data || !offsets || !sizes || n_streams < 1 || tile_width < 1 || tile_height < 1)
        return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "decodeLosslessJPEG: null buffer or no streams");
    const int tiles_across = (out->width + tile_width - 1) / tile_width;
    size_t span0 = ~(size_t)0, span1 = 0;
    for (int i = 0; i < n_streams; i++) {
        if (offsets[i] > data_size || sizes[i] > data_size - offsets[i] || sizes[i] < 4)
            return set_error(ctx, GLS_ERR_INVALID_ARGUMENT, "decodeLosslessJPEG: stream %d outside the buffer", i);
        span0 = std::min(span0, (size_t)offsets[i]);
        span1 = std::max(span1, (size_t)(offsets[i] + sizes[i]));
    }

    // parse every stream; lay out intervals, chunks, segments and rows
    std::vector<LjStream> streams(n_streams);
    std::vector<LjInterval> intervals;
    std::vector<LjChunk> chunks;
    std::vector<LjTable> tables;
    std::vector<int> seg_interval, row_stream;
    long long samples = 0, dst_bytes = 0;
    for (int i = 0; i < n_streams; i++) {
        const uint8_t* d = data + offsets[i];
        const size_t n = sizes[i];
        HostHeader h;
        if (!parse_header(d, n, h))
            return set_error(ctx, GLS_ERR_BAD_STREAM, "decodeLosslessJPEG: stream %d: malformed header", i);
        if ((long long)h.width * h.height * h.ns != (long long)tile_width * tile_height)
            return set_error(ctx, GLS_ERR_BAD_STREAM,
                             "decodeLosslessJPEG: stream %d decodes to %dx%dx%d samples, the tile holds %dx%d", i,
                             h.width, h.height, h.ns, tile_width, tile_height);
        LjStream& st = streams[i];
        st.width = h.width;
        st.height = h.height;
        st.comps = h.ns;
        st.precision = h.precision;
        st.predictor = h.ss;
        st.pt = h.pt;
        for (int k = 0; k < 4; k++) {
            if (k >= h.ns) {
                st.table[k] = st.table[0];
                continue;
            }
            st.table[k] = (int)tables.size();
            LjTable t;
            derive_table(h.tab[h.scan_table[k]], t);
            tables.push_back(t);
        }
        // decode unit: a single codeword when the scan's tables all parse bits alike
        bool alike = true;
        for (int k = 1; k < h.ns; k++) alike = alike && same_parse(h.tab[h.scan_table[0]], h.tab[h.scan_table[k]]);
        st.upc = alike ? 1 : h.ns;
        // a unit whose codewords are all zero bits and all decode to category 0
        st.zero_unit_bits = 0;
        for (int k = 0; k < h.ns; k++) {
            const uint16_t lk = tables[st.table[k]].look[0];
            if (lk == 0 || (lk & 0xFF) != 0) {
                st.zero_unit_bits = 0;
                break;
            }
            if (k < st.upc) st.zero_unit_bits += lk >> 8;
        }
        // QuickPredict throws for a predictor above 7 once a row is predicted from the one
        // above (gls_dng_lossless_jpeg.cpp:1290); the first row's 2^(P-Pt-1) needs Pt < P
        const int rows_per_restart = h.restart / h.width;
        if (h.ss > 7 && h.width > 1 && h.height > 1 && rows_per_restart != 1)
            return set_error(ctx, GLS_ERR_BAD_STREAM, "decodeLosslessJPEG: stream %d: predictor %d", i, h.ss);
        st.sample_off = samples;
        samples += (long long)h.width * h.height * h.ns;
        st.tile_w = tile_width;
        st.tile_x = tile_width * (i % tiles_across);
        st.tile_y = tile_height * (i / tiles_across);
        if (st.tile_x >= out->width || st.tile_y >= out->height)
            return set_error(ctx, GLS_ERR_INVALID_SIZE, "decodeLosslessJPEG: tile %d lies outside the image", i);
        st.clip_w = std::min(st.tile_x + tile_width, out->width) - st.tile_x;
        st.clip_h = std::min(st.tile_y + tile_height, out->height) - st.tile_y;
        st.row_base = (int)row_stream.size();
        for (int r = 0; r < h.height; r++) row_stream.push_back(i);
        st.interval_base = (int)intervals.size();
        // restart intervals: rows per interval, each interval's data ends at its marker
        const int rr = h.restart / h.width;
        const int nint = rr > 0 ? (h.height + rr - 1) / rr : 1;
        size_t pos = h.scan_pos;
        for (int k = 0; k < nint; k++) {
            LjInterval iv;
            iv.stream = i;
            iv.first_row = rr > 0 ? k * rr : 0;
            iv.rows = rr > 0 ? std::min(rr, h.height - k * rr) : h.height;
            iv.mcu_off = (long long)iv.first_row * h.width;
            iv.src_begin = (long long)(offsets[i] + pos - span0);
            size_t lim = n;
            if (k + 1 < nint) {  // find the marker that ends this interval and check it is RSTk
                size_t q = pos;
                while (q + 1 < n && !(d[q] == 0xFF && d[q + 1] != 0)) q++;
                if (q + 1 >= n)
                    return set_error(ctx, GLS_ERR_BAD_STREAM, "decodeLosslessJPEG: stream %d: restart marker missing", i);
                size_t r = q + 1;
                while (r < n && d[r] == 0xFF) r++;
                if (r >= n || d[r] != 0xD0 + (k & 7))
                    return set_error(ctx, GLS_ERR_BAD_STREAM, "decodeLosslessJPEG: stream %d: bad restart marker", i);
                lim = q;
                pos = r + 1;
            }
            iv.src_limit = (long long)(offsets[i] + lim - span0);
            if (k + 1 == nint) iv.src_limit = (long long)(offsets[i] + n - span0);
            const long long len = std::max(0ll, iv.src_limit - iv.src_begin);
            iv.dst_off = dst_bytes;
            iv.dst_words = (len + kPad + 3) / 4 + 2;
            dst_bytes += iv.dst_words * 4;
            iv.chunk_base = (int)chunks.size();
            for (long long b = iv.src_begin; b < iv.src_limit; b += kChunk)
                chunks.push_back(LjChunk{b, std::min(b + kChunk, iv.src_limit), (int)intervals.size()});
            iv.nchunk = (int)chunks.size() - iv.chunk_base;
            iv.seg_base = (int)seg_interval.size();
            iv.nseg = (int)std::max(1ll, (len * 8 + kSegBits - 1) / kSegBits);
            for (int j = 0; j < iv.nseg; j++) seg_interval.push_back((int)intervals.size());
            intervals.push_back(iv);
        }
        st.nint = nint;
    }
    const int nint = (int)intervals.size(), nchunk = (int)chunks.size(), nseg = (int)seg_interval.size();
    const int nrows = (int)row_stream.size();
    const size_t span = span1 - span0;

    // device scratch
    size_t off = 0;
    const size_t o_src = carve<uint8_t>(off, span + 8);
    const size_t o_dst = carve<uint8_t>(off, (size_t)dst_bytes + 16);
    const size_t o_str = carve<LjStream>(off, n_streams);
    const size_t o_int = carve<LjInterval>(off, nint);
    const size_t o_chk = carve<LjChunk>(off, std::max(nchunk, 1));
    const size_t o_tab = carve<LjTable>(off, tables.size());
    const size_t o_segi = carve<int>(off, nseg);
    const size_t o_rows = carve<int>(off, nrows);
    const size_t o_mark = carve<unsigned long long>(off, nint);
    const size_t o_dlen = carve<long long>(off, nint);
    const size_t o_cst = carve<int>(off, std::max(nchunk, 1));
    const size_t o_coff = carve<long long>(off, std::max(nchunk, 1));
    const size_t o_su = carve<long long>(off, nseg);
    const size_t o_bnd = carve<long long>(off, (size_t)nseg * kBnd);
    const size_t o_p1c = carve<int>(off, nseg);
    const size_t o_p1 = carve<int8_t>(off, nseg);
    const size_t o_ea = carve<long long>(off, nseg);
    const size_t o_eb = carve<long long>(off, nseg);
    const size_t o_cnt = carve<int>(off, nseg);
    const size_t o_soff = carve<long long>(off, nseg);
    const size_t o_flags = carve<int>(off, 4);
    const size_t o_diff = carve<int16_t>(off, (size_t)samples);
    const size_t o_rec = carve<uint16_t>(off, (size_t)samples);
    GLS_CHECK(ensure_scratch(ctx, off + 256));
    char* S = (char*)ctx->scratch;
    cudaStream_t cs = ctx->stream;

    std::vector<unsigned long long> marks(nint);
    for (int k = 0; k < nint; k++) marks[k] = (unsigned long long)intervals[k].src_limit;
    GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(S + o_src, data + span0, span, cudaMemcpyHostToDevice, cs), "copy streams"));
    GLS_CHECK(check_cuda(ctx, cudaMemsetAsync(S + o_dst, 0, (size_t)dst_bytes + 16, cs), "clear"));
    GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(S + o_str, streams.data(), n_streams * sizeof(LjStream), cudaMemcpyHostToDevice, cs), "copy"));
    GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(S + o_int, intervals.data(), nint * sizeof(LjInterval), cudaMemcpyHostToDevice, cs), "copy"));
    if (nchunk)
        GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(S + o_chk, chunks.data(), nchunk * sizeof(LjChunk), cudaMemcpyHostToDevice, cs), "copy"));
    GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(S + o_tab, tables.data(), tables.size() * sizeof(LjTable), cudaMemcpyHostToDevice, cs), "copy"));
    GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(S + o_segi, seg_interval.data(), nseg * sizeof(int), cudaMemcpyHostToDevice, cs), "copy"));
    GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(S + o_rows, row_stream.data(), nrows * sizeof(int), cudaMemcpyHostToDevice, cs), "copy"));
    GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(S + o_mark, marks.data(), nint * sizeof(unsigned long long), cudaMemcpyHostToDevice, cs), "copy"));
    GLS_CHECK(check_cuda(ctx, cudaMemsetAsync(S + o_flags, 0, 4 * sizeof(int), cs), "clear flags"));
    // the source span is followed by 8 readable bytes (a marker test looks one byte ahead)
    GLS_CHECK(check_cuda(ctx, cudaMemsetAsync(S + o_src + span, 0xFF, 8, cs), "pad"));

    LjDev g;
    g.src = (const uint8_t*)(S + o_src);
    g.dst = (uint8_t*)(S + o_dst);
    g.streams = (const LjStream*)(S + o_str);
    g.intervals = (const LjInterval*)(S + o_int);
    g.chunks = (const LjChunk*)(S + o_chk);
    g.tables = (const LjTable*)(S + o_tab);
    g.seg_interval = (const int*)(S + o_segi);
    g.row_stream = (const int*)(S + o_rows);
    g.marker = (unsigned long long*)(S + o_mark);
    g.dlen = (long long*)(S + o_dlen);
    g.chunk_stuff = (int*)(S + o_cst);
    g.chunk_off = (long long*)(S + o_coff);
    g.start_used = (long long*)(S + o_su);
    g.bnd = (long long*)(S + o_bnd);
    g.p1cnt = (int*)(S + o_p1c);
    g.p1 = (int8_t*)(S + o_p1);
    g.end_a = (long long*)(S + o_ea);
    g.end_b = (long long*)(S + o_eb);
    g.cnt = (int*)(S + o_cnt);
    g.seg_off = (long long*)(S + o_soff);
    g.error = (int*)(S + o_flags);
    g.diff = (int16_t*)(S + o_diff);
    g.recon = (uint16_t*)(S + o_rec);
    g.out = (uint16_t*)out->ptr;
    g.out_pitch = pitch_elems(out);

    if (nchunk) {
        lj_marker_kernel<<<nchunk, 256, 0, cs>>>(g);
        lj_stuff_count_kernel<<<nchunk, 256, 0, cs>>>(g);
    }
    lj_chunk_offsets_kernel<<<nint, 256, 0, cs>>>(g);
    if (nchunk) lj_destuff_kernel<<<nchunk, 256, 0, cs>>>(g);
    ctx->launches += nchunk ? 4 : 1;
    const int sb = 128, sg = (nseg + sb - 1) / sb;
    lj_phase1_kernel<<<sg, sb, 0, cs>>>(g, nseg);
    ctx->launches++;
    long long* e_in = g.end_a;
    long long* e_out = g.end_b;
    for (int round = 0; round < kSyncRounds; round++) {
        lj_sync_kernel<<<sg, sb, 0, cs>>>(g, nseg, e_in, e_out);
        std::swap(e_in, e_out);
    }
    lj_repair_kernel<<<sg, sb, 0, cs>>>(g, nseg, e_in, e_out);
    std::swap(e_in, e_out);
    lj_walk_kernel<<<nint, 256, 0, cs>>>(g, e_in, (int*)e_out);  // the other end buffer holds the lists
    ctx->launches += kSyncRounds + 2;
    lj_count_scan_kernel<<<nint, 256, 0, cs>>>(g);
    lj_write_kernel<<<sg, sb, 0, cs>>>(g, nseg);
    lj_col0_kernel<<<nint * 4, 256, 0, cs>>>(g);
    lj_row_scan_kernel<<<nrows, 256, 0, cs>>>(g, nrows);
    lj_rows_general_kernel<<<nint, 256, 0, cs>>>(g, nint);
    lj_place_kernel<<<nrows, 256, 0, cs>>>(g, nrows);
    ctx->launches += 6;
    GLS_CHECK(check_launch(ctx, "decodeLosslessJPEG"));
    int* h_flag = (int*)ctx->host_pinned;
    GLS_CHECK(check_cuda(ctx, cudaMemcpyAsync(h_flag, g.error, sizeof(int), cudaMemcpyDeviceToHost, cs), "flag"));
    GLS_CHECK(check_cuda(ctx, cudaStreamSynchronize(cs), "synchronize"));
    if (*h_flag) return set_error(ctx, GLS_ERR_BAD_STREAM, "decodeLosslessJPEG: a difference category above 16");
    return GLS_OK;
}
