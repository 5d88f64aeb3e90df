// Greedy max clique on a bit-packed adjacency (sm_103a).
//
// Exact replica of FMC::maxCliqueHeu / maxCliqueHeuIncremental
// (include/KimeraRPGO/max_clique_finder/findCliqueHeu.cpp:32-209) as called by
// findMaxCliqueHeu[Incremental] (src/utils/GraphUtils.cpp:19-44):
//  * candidate v is skipped when the running best exceeds deg(v);
//  * its work list is [v] followed by its neighbours u (ascending) with
//    deg(u) >= best;
//  * every round takes the last list element m and keeps, in order, the
//    elements adjacent to m (with deg >= best); the number of rounds is the
//    candidate's score;
//  * a candidate that beats the running best copies the whole work buffer.
// Because every kept element after the first is a neighbour of v and the list
// stays sorted, the list is [v] + a set B, m = max(B) and B' = B & N(m): each
// round is one AND of bit rows plus a population count. The buffer slot p > 0
// ends up holding the p-th smallest element of the last round's B with at
// least p elements, so a round that shrinks B from n_r to n_{r+1} elements
// writes its n_r - n_{r+1} largest elements to slots (n_{r+1}, n_r].
//
// The running best makes candidates depend on each other only through the
// pruning threshold, so a window of candidates is scored concurrently with
// the threshold at the window start; the host takes the first candidate that
// improves and restarts the window after it (later results used a stale
// threshold). A candidate that can no longer beat the threshold
// (rounds + |B| + 1 <= best) stops early: it could not change the result.
// Each round waits on one adjacency row (that of m); the row of B's
// second-highest element, the next round's m whenever it is adjacent to m
// (most rounds on dense matrices), is fetched one round ahead.
// Clean runs: a round whose m is adjacent to every element of B below it
// only removes m, so the next round's m is B's next element, known before
// the round. Rounds are therefore taken in batches: the rows of B's 32
// highest elements u_0 > u_1 > ... are checked against B (one row per lane,
// all 32 in flight) and the leading run of clean ones is committed at
// once (B loses those elements; each goes to the slot of its round); the
// first element that is not clean takes an ordinary round.
#include <mutex>

#include "../../include/rpgo_gb300.h"
#include "pcm_kernels.hpp"

namespace rpgo {
namespace {

__global__ void k_degrees(int n, const uint32_t* __restrict__ adj, int words, int32_t* __restrict__ deg) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n) return;
  int c = 0;
  for (int w = lane; w < words; w += 32) {
    uint32_t x = adj[(size_t)warp * words + w];
    if (32 * w + 32 > n) x &= (32 * w >= n) ? 0u : ((1u << (n - 32 * w)) - 1u);  // ignore padding bits
    if (w == (warp >> 5)) x &= ~(1u << (warp & 31));                               // and the diagonal
    c += __popc(x);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if (lane == 0) deg[warp] = c;
}

__device__ __forceinline__ int warp_sum(int v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_max(int v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

constexpr int kRowRegs = 24;  // register words per lane of a prefetched adjacency row (n <= 24,576)
constexpr int kWindowThreads = 256;  // block of k_clique_window: 8 candidates

// One warp per candidate of the window [v0, v0 + count).
// result[s]: -1 pruned (deg < best), -2 cannot beat best, else icc.
// sets: per slot 2*words (double buffer); bufs: per slot buf_len ints.
__global__ void k_clique_window(int n, const uint32_t* __restrict__ adj, int words, const int32_t* __restrict__ deg,
                                int v0, int count, int best, int32_t* __restrict__ result,
                                uint32_t* __restrict__ sets, int32_t* __restrict__ bufs, int buf_len) {
  __shared__ int sh_top[kWindowThreads / 32][32];
  __shared__ __align__(16) uint32_t sh_b[kWindowThreads / 32][32 * kRowRegs];
  const int slot = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (slot >= count) return;
  int* const top32 = sh_top[threadIdx.x >> 5];
  uint32_t* const bsh = sh_b[threadIdx.x >> 5];
  const int v = v0 + slot;
  if (best > deg[v]) {
    if (lane == 0) result[slot] = -1;
    return;
  }
  uint32_t* cur = sets + (size_t)slot * 2 * words;
  uint32_t* nxt = cur + words;
  int32_t* buf = bufs + (size_t)slot * buf_len;
  // B0 = N(v) restricted to deg >= best
  int cnt = 0, top = -1;
  for (int w = lane; w < words; w += 32) {
    uint32_t x = adj[(size_t)v * words + w];
    uint32_t keep = 0;
    while (x) {
      const int b = __ffs(x) - 1;
      x &= x - 1;
      const int u = 32 * w + b;
      if (u < n && u != v && best <= deg[u]) keep |= 1u << b;
    }
    cur[w] = keep;
    cnt += __popc(keep);
    if (keep) top = w;
  }
  int nr = warp_sum(cnt);
  top = warp_max(top);
  if (lane == 0) buf[0] = v;
  int r = 0;
  // rows of at most 32 * kRowRegs words are held in registers: the row of
  // this round's m and the prefetched row of the likely next one. Only the
  // first ceil(n / 32) words of a row can hold bits (the row stride `words`
  // may be a larger capacity)
  const bool regs = (n + 31) / 32 <= 32 * kRowRegs;
  const bool vec = (words & 3) == 0 && (reinterpret_cast<uintptr_t>(adj) & 15) == 0;
  uint32_t row[kRowRegs], pf[kRowRegs];
  int pf_m = -1;
  // clean-run batches are tried from round try_at on; after a batch whose
  // first element was not clean, the next try waits 2, 4, ... 64 rounds
  int try_at = 0, misses = 0;
  __syncwarp();
  while (true) {
    if (nr == 0) {
      if (lane == 0) result[slot] = r + 1;
      return;
    }
    if (r + nr + 1 <= best) {
      if (lane == 0) result[slot] = -2;
      return;
    }
    if (regs && r >= try_at) {
      // B's (up to) 32 highest elements, descending, into top32
      int n_top = 0;
      for (int base = top; base >= 0 && n_top < 32; base -= 32) {
        const int w = base - lane;  // lane 0 takes the highest word of the chunk
        const uint32_t x = (w >= 0) ? cur[w] : 0u;
        const int pc = __popc(x);
        int incl = pc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += y;
        }
        uint32_t y = x;
        int q = n_top + incl - pc;
        while (y && q < 32) {
          const int b = 31 - __clz(y);
          y &= ~(1u << b);
          top32[q++] = 32 * w + b;
        }
        n_top += __shfl_sync(0xffffffffu, incl, 31);
      }
      n_top = min(n_top, 32);
      __syncwarp();
      // B's words into shared memory; u_l is clean when B's elements below
      // u_l are all in N(u_l) (the rounds before it, clean, removed exactly
      // the elements above it)
      const int u0 = top32[0];
      const int wmax = u0 >> 5;
      for (int w = lane; w <= wmax; w += 32) bsh[w] = cur[w];
      __syncwarp();
      // lane l checks u_l on its own row, 32 words (one line) per step, the
      // lines two steps ahead prefetched into L1; every lane reads B's words
      // from shared memory (broadcast). Steps below every lane's last word
      // need no mask; in the others, loads past u_l's word are clamped to it
      // and masked out. An empty lane checks u_0's row (its verdict is unused).
      const int u = lane < n_top ? top32[lane] : -1;
      const int ue = u >= 0 ? u : u0;
      const int wl = ue >> 5;
      const uint32_t low = (1u << (ue & 31)) - 1u;
      const uint32_t* const rp = adj + (size_t)ue * words;
      uint32_t viol = 0u;
      if (vec) {
        const uint4* const rp4 = reinterpret_cast<const uint4*>(rp);
        const uint4* const b4 = reinterpret_cast<const uint4*>(bsh);
#pragma unroll
        for (int q = 0; q < kRowRegs; ++q) {
          if (32 * q > wmax) break;
          if (32 * q + 64 <= wl) asm volatile("prefetch.global.L1 [%0];" ::"l"(rp + 32 * q + 64));
          if (__all_sync(0xffffffffu, 32 * q + 31 < wl)) {
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const uint4 r4 = __ldg(rp4 + 8 * q + j);
              const uint4 bb = b4[8 * q + j];
              viol |= (bb.x & ~r4.x) | (bb.y & ~r4.y) | (bb.z & ~r4.z) | (bb.w & ~r4.w);
            }
          } else {
            uint4 rw[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) rw[j] = __ldg(rp4 + (min(32 * q + 4 * j, wl & ~3) >> 2));
#pragma unroll
            for (int j = 0; j < 8; ++j) {
              const uint4 bb = b4[8 * q + j];
              const uint32_t e[4] = {rw[j].x, rw[j].y, rw[j].z, rw[j].w};
              const uint32_t f[4] = {bb.x, bb.y, bb.z, bb.w};
#pragma unroll
              for (int t = 0; t < 4; ++t) {
                const int w = 32 * q + 4 * j + t;
                const uint32_t msk = w < wl ? 0xffffffffu : (w == wl ? low : 0u);
                viol |= f[t] & msk & ~e[t];
              }
            }
          }
          // u_0 not clean: nothing to commit, the next round is an ordinary one
          if (__shfl_sync(0xffffffffu, viol, 0) != 0u) break;
        }
      } else {
#pragma unroll
        for (int q = 0; q < kRowRegs; ++q) {
          if (32 * q > wmax) break;
          if (32 * q + 64 <= wl) asm volatile("prefetch.global.L1 [%0];" ::"l"(rp + 32 * q + 64));
          uint32_t rw[32];
#pragma unroll
          for (int j = 0; j < 32; ++j) rw[j] = __ldg(rp + min(32 * q + j, wl));
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int w = 32 * q + j;
            const uint32_t msk = w < wl ? 0xffffffffu : (w == wl ? low : 0u);
            viol |= bsh[w] & msk & ~rw[j];
          }
          if (__shfl_sync(0xffffffffu, viol, 0) != 0u) break;
        }
      }
      const unsigned bad = __ballot_sync(0xffffffffu, u < 0 || viol != 0u);
      const int k = bad ? __ffs(bad) - 1 : 32;  // leading clean elements
      if (k > 0) {
        // rounds r .. r+k-1: B shrinks by its highest element, which goes to
        // the slot of the round (B's size then)
        for (int l = lane; l < k; l += 32) buf[nr - l] = top32[l];
        const int ul = top32[k - 1];
        __syncwarp();
        if (lane == 0) cur[ul >> 5] &= (1u << (ul & 31)) - 1u;  // words above top are never read
        top = ul >> 5;
        nr -= k;
        r += k;
        pf_m = -1;
        misses = 0;
        // a batch that stopped early stopped at an element that is not clean:
        // the next round is an ordinary one
        try_at = k < n_top ? r + 1 : r;
        __syncwarp();
        continue;
      }
      misses = min(misses + 1, 6);
      try_at = r + (1 << misses);
    }
    // m = highest element of B: top word's highest bit
    int m;
    {
      // find the highest nonzero word at or below `top`
      int hw = -1;
      for (int base = top - (top % 32); base >= 0 && hw < 0; base -= 32) {
        const int w = base + lane;
        const uint32_t x = (w <= top && w < words) ? cur[w] : 0u;
        const unsigned msk = __ballot_sync(0xffffffffu, x != 0u);
        if (msk) {
          const int l = 31 - __clz(msk);
          hw = base + l;
        }
      }
      if (hw < 0) {  // cannot happen when nr > 0; never index below the set
        if (lane == 0) result[slot] = -3;
        return;
      }
      top = hw;
      const uint32_t xw = cur[hw];
      m = 32 * hw + (31 - __clz(xw));
    }
    // B' = B & N(m) over words [0, top]
    int c2 = 0, top2 = -1;
    if (regs) {
      // row of m from the registers when the previous round fetched it
      if (pf_m != m) {
#pragma unroll
        for (int q = 0; q < kRowRegs; ++q) {
          const int w = lane + 32 * q;
          row[q] = (w <= top) ? adj[(size_t)m * words + w] : 0u;
        }
      } else {
#pragma unroll
        for (int q = 0; q < kRowRegs; ++q) row[q] = pf[q];
      }
      // fetch the row of B's second-highest element, the next m whenever it
      // is a neighbour of m (its words up to the current top cover every
      // later round's, as top only falls); read by the next round
      uint32_t below = cur[top] & ~(1u << (m & 31));
      int m2 = below ? 32 * top + (31 - __clz(below)) : -1;
      if (m2 < 0 && top > 0) {
        const int w = top - 1 - lane;
        const uint32_t x = (w >= 0) ? cur[w] : 0u;
        const unsigned msk = __ballot_sync(0xffffffffu, x != 0u);
        if (msk) {
          const int l = __ffs(msk) - 1;  // lowest lane = highest word
          const uint32_t xl = __shfl_sync(0xffffffffu, x, l);
          m2 = 32 * (top - 1 - l) + (31 - __clz(xl));
        }
      }
      pf_m = m2;
      if (m2 >= 0) {
#pragma unroll
        for (int q = 0; q < kRowRegs; ++q) {
          const int w = lane + 32 * q;
          pf[q] = (w <= top) ? adj[(size_t)m2 * words + w] : 0u;
        }
      }
#pragma unroll
      for (int q = 0; q < kRowRegs; ++q) {
        const int w = lane + 32 * q;
        if (w <= top) {
          uint32_t x = cur[w] & row[q];
          if (w == (m >> 5)) x &= ~(1u << (m & 31));  // m is never its own neighbour: every round shrinks B
          nxt[w] = x;
          c2 += __popc(x);
          if (x) top2 = w;
        }
      }
    } else {
      for (int w = lane; w <= top; w += 32) {
        uint32_t x = cur[w] & adj[(size_t)m * words + w];
        if (w == (m >> 5)) x &= ~(1u << (m & 31));  // m is never its own neighbour: every round shrinks B
        nxt[w] = x;
        c2 += __popc(x);
        if (x) top2 = w;
      }
    }
    const int n_next = warp_sum(c2);
    top2 = warp_max(top2);
    __syncwarp();
    // slots (n_next, nr] <- the nr - n_next largest elements of B, ascending
    int need = nr - n_next;
    int pos = nr;  // slot of the next element taken from the top
    for (int base = top; base >= 0 && need > 0; base -= 32) {
      const int w = base - lane;  // lane 0 takes the highest word of the chunk
      const uint32_t x = (w >= 0) ? cur[w] : 0u;
      const int pc = __popc(x);
      // exclusive prefix from the top (lane 0 first)
      int incl = pc;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const int excl = incl - pc;
      if (excl < need) {
        // emit elements of this word from its top bit down
        uint32_t y = x;
        int q = excl;
        while (y && q < need) {
          const int b = 31 - __clz(y);
          y &= ~(1u << b);
          buf[pos - q] = 32 * w + b;
          ++q;
        }
      }
      const int total = __shfl_sync(0xffffffffu, incl, 31);
      need -= total;
      pos -= total;
    }
    __syncwarp();
    uint32_t* t = cur;
    cur = nxt;
    nxt = t;
    nr = n_next;
    top = top2 < 0 ? 0 : top2;
    ++r;
  }
}

}  // namespace

int max_clique_heu(int n, const uint32_t* adj, int words, int first, int seed, std::vector<int32_t>* clique,
                   CliqueWorkspace& ws, cudaStream_t st) {
  clique->clear();
  if (n <= 0) return seed;
  ws.deg.resize(n);
  {
    const int tb = 256;
    k_degrees<<<div_up((int64_t)n * 32, tb), tb, 0, st>>>(n, adj, words, ws.deg.get());
    RPGO_LAUNCHED();
  }
  const int W = 2048;
  const int buf_len = n + 1;
  ws.result.resize(W);
  ws.sets.resize((size_t)W * 2 * words);
  ws.buffers.resize((size_t)W * buf_len);
  ws.h_result.resize(W);
  int best = seed;
  int best_slot_v = -1;
  std::vector<int32_t> best_buf;
  int v = std::max(first, 0);
  while (v < n) {
    const int count = std::min(W, n - v);
    const int tb = kWindowThreads;
    k_clique_window<<<div_up((int64_t)count * 32, tb), tb, 0, st>>>(n, adj, words, ws.deg.get(), v, count, best,
                                                                    ws.result.get(), ws.sets.get(),
                                                                    ws.buffers.get(), buf_len);
    RPGO_LAUNCHED();
    ws.result.download(ws.h_result.data(), count, st);
    RPGO_CUDA(cudaStreamSynchronize(st));
    int improved = -1;
    for (int s = 0; s < count; ++s)
      if (ws.h_result[s] > best) {
        improved = s;
        break;
      }
    if (improved < 0) {
      v += count;
      continue;
    }
    best = ws.h_result[improved];
    best_slot_v = v + improved;
    best_buf.resize(best);
    RPGO_CUDA(cudaMemcpyAsync(best_buf.data(), ws.buffers.get() + (size_t)improved * buf_len,
                              sizeof(int32_t) * best, cudaMemcpyDeviceToHost, st));
    RPGO_CUDA(cudaStreamSynchronize(st));
    v = v + improved + 1;
  }
  (void)best_slot_v;
  *clique = best_buf;
  return best;
}

}  // namespace rpgo

// ---------------------------------------------------------------------------
// Allocation-free variant: the same two kernels and window loop, with every
// device work array carved out of one file-scope scratch array instead of
// cudaMalloc'd buffers. Limits: n <= RPGO_CLIQUE_NOALLOC_MAX_N closures,
// row stride words <= RPGO_CLIQUE_NOALLOC_MAX_WORDS, and a window of
// kNoAllocWindow candidates (the result does not depend on the window size:
// the host always continues after the first improving candidate).
namespace rpgo {
namespace {

constexpr int kNoAllocWindow = 128;
constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }
// Region offsets (bytes) inside the scratch array.
constexpr size_t kDegOff = 0;
constexpr size_t kResultOff = kDegOff + align_up(sizeof(int32_t) * RPGO_CLIQUE_NOALLOC_MAX_N);
constexpr size_t kSetsOff = kResultOff + align_up(sizeof(int32_t) * kNoAllocWindow);
constexpr size_t kBufsOff =
    kSetsOff + align_up(sizeof(uint32_t) * (size_t)kNoAllocWindow * 2 * RPGO_CLIQUE_NOALLOC_MAX_WORDS);
constexpr size_t kScratchBytes =
    kBufsOff + align_up(sizeof(int32_t) * (size_t)kNoAllocWindow * (RPGO_CLIQUE_NOALLOC_MAX_N + 1));
static_assert(kScratchBytes == RPGO_CLIQUE_NOALLOC_SCRATCH_BYTES, "scratch size in the header is stale");

// Held by every device that loads this library, until the process exits.
// In host code `g_clique_scratch` is only a handle for cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_clique_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device; looked up once
// per device (the first call on a device) with that device current. The
// address belongs to the device's primary context: after cudaDeviceReset the
// cached address is stale, so this entry point must not be used again in that
// process.
int scratch_for_current_device(unsigned char** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return RPGO_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    unsigned char* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void**)&ptr, g_clique_scratch);
    if (e != cudaSuccess || !ptr) {
      std::fprintf(stderr, "rpgo_gb300: cudaGetSymbolAddress(clique scratch) failed: %s\n", cudaGetErrorString(e));
      return RPGO_ERR_CUDA;
    }
    g_scratch_ptr[dev] = ptr;
  }
  *out = g_scratch_ptr[dev];
  return RPGO_OK;
}

int max_clique_heu_noalloc(int n, const uint32_t* adj, int words, int first, int seed, int32_t* clique_out,
                           int32_t* size_out, unsigned char* scratch, cudaStream_t st) {
  int32_t* deg = reinterpret_cast<int32_t*>(scratch + kDegOff);
  int32_t* result = reinterpret_cast<int32_t*>(scratch + kResultOff);
  uint32_t* sets = reinterpret_cast<uint32_t*>(scratch + kSetsOff);
  int32_t* bufs = reinterpret_cast<int32_t*>(scratch + kBufsOff);
  int best = seed;
  if (n > 0) {
    // The array keeps the previous call's contents. Only the window results
    // are cleared here; deg, the candidate sets and the work buffers are
    // written by the kernels before they are read.
    RPGO_CUDA(cudaMemsetAsync(result, 0, sizeof(int32_t) * kNoAllocWindow, st));
    {
      const int tb = 256;
      k_degrees<<<div_up((int64_t)n * 32, tb), tb, 0, st>>>(n, adj, words, deg);
      RPGO_LAUNCHED();
    }
    const int buf_len = n + 1;
    int32_t h_result[kNoAllocWindow];
    int v = std::max(first, 0);
    while (v < n) {
      const int count = std::min(kNoAllocWindow, n - v);
      const int tb = kWindowThreads;
      k_clique_window<<<div_up((int64_t)count * 32, tb), tb, 0, st>>>(n, adj, words, deg, v, count, best, result,
                                                                      sets, bufs, buf_len);
      RPGO_LAUNCHED();
      RPGO_CUDA(cudaMemcpyAsync(h_result, result, sizeof(int32_t) * count, cudaMemcpyDeviceToHost, st));
      RPGO_CUDA(cudaStreamSynchronize(st));
      int improved = -1;
      for (int s = 0; s < count; ++s)
        if (h_result[s] > best) {
          improved = s;
          break;
        }
      if (improved < 0) {
        v += count;
        continue;
      }
      best = h_result[improved];
      // The winner's work buffer goes straight to the caller's output; a
      // later, larger winner overwrites it.
      if (clique_out) {
        RPGO_CUDA(cudaMemcpyAsync(clique_out, bufs + (size_t)improved * buf_len, sizeof(int32_t) * best,
                                  cudaMemcpyDeviceToHost, st));
        RPGO_CUDA(cudaStreamSynchronize(st));
      }
      v = v + improved + 1;
    }
  }
  *size_out = best;
  return RPGO_OK;
}

}  // namespace
}  // namespace rpgo

extern "C" int rpgo_max_clique_heu_dev_noalloc(int32_t n, const uint32_t* adj, int32_t words, int32_t first,
                                               int32_t seed, int32_t* clique_out, int32_t* size_out,
                                               void* stream) {
  if (n < 0 || words < (n + 31) / 32 || !size_out || (n > 0 && !adj)) return RPGO_ERR_ARG;
  if (n > RPGO_CLIQUE_NOALLOC_MAX_N || words > RPGO_CLIQUE_NOALLOC_MAX_WORDS) {
    std::fprintf(stderr,
                 "rpgo_gb300: rpgo_max_clique_heu_dev_noalloc: n = %d, words = %d exceeds the fixed scratch "
                 "(n <= %d, words <= %d)\n",
                 (int)n, (int)words, RPGO_CLIQUE_NOALLOC_MAX_N, RPGO_CLIQUE_NOALLOC_MAX_WORDS);
    return RPGO_ERR_SIZE;
  }
  try {
    unsigned char* scratch = nullptr;
    const int rc = rpgo::scratch_for_current_device(&scratch);
    if (rc != RPGO_OK) return rc;
    return rpgo::max_clique_heu_noalloc(n, adj, words, first, seed, clique_out, size_out, scratch,
                                        (cudaStream_t)stream);
  } catch (const rpgo::CudaError& e) {
    std::fprintf(stderr, "rpgo_gb300: %s\n", e.what());
    return RPGO_ERR_CUDA;
  } catch (...) {
    // nothing may cross the C ABI (a failed mutex lock throws std::system_error)
    std::fprintf(stderr, "rpgo_gb300: rpgo_max_clique_heu_dev_noalloc: unexpected exception\n");
    return RPGO_ERR_CUDA;
  }
}
