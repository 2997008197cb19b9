// The process's libc rand() sequence, drawn in bulk.
//
// The drop-in sweep needs one rand() per sub-segment in traversal order, as
// the serial reference draws them (src/solver.c:476-483): tens of millions of
// calls per sweep, each taking libc's lock.  glibc's rand() is its random():
// for the state types 1-4 an additive lagged-Fibonacci generator over the
// ring of the state buffer,
//     x_k = x_{k-deg} + x_{k-sep}  (mod 2^32),   rand() = x_k >> 1,
// with (deg, sep) = (7, 3), (15, 1), (31, 3) (the default state) and (63, 1)
// (glibc stdlib/random_r.c, the generator of BSD 4.3 random(3)).  The state
// buffer that initstate()/setstate() exchange holds one header word,
// 5 * rear + type, and the ring; setstate() writes the current position into
// the header of the state it leaves and returns that buffer.
//
// moc_libc_draws() swaps a scratch state in with setstate(), reads the
// process's ring and position from the buffer it got back, produces the next
// n values of the sequence with the recurrence, writes the advanced ring and
// position back and swaps the state in again: libc then continues exactly
// where n rand() calls would have left it.  Once per process the bulk path is
// checked against real rand() calls on a scratch state; if the check fails,
// the library is not glibc, or the process uses the type-0 linear
// congruential state, every value comes from rand() itself.  Like the serial
// reference, this assumes no other thread calls rand() meanwhile.
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

#include <algorithm>
#include <mutex>
#include <vector>

namespace {

constexpr int MAX_TYPES = 5;
constexpr int DEG[MAX_TYPES] = {0, 7, 15, 31, 63};
constexpr int SEP[MAX_TYPES] = {0, 3, 1, 3, 1};     // 3 or 1: the loops below rely on it

// count values of the recurrence from the window x[0..deg) (oldest first),
// into out; the window then holds the last deg values
void lfg_run(uint32_t *win, int deg, int sep, int32_t *out, int64_t count) {
  constexpr int64_t CH = 16384;
  std::vector<uint32_t> w((size_t)(deg + CH));
  memcpy(w.data(), win, sizeof(uint32_t) * (size_t)deg);
  for (int64_t done = 0; done < count;) {
    const int64_t c = std::min<int64_t>(CH, count - done);
    uint32_t *__restrict x = w.data();
    int32_t *__restrict o = out + done;
    if (sep == 3) {
      // the short lag from registers: x_{k-3}, x_{k-2}, x_{k-1}
      uint32_t a = x[deg - 3], b = x[deg - 2], d = x[deg - 1];
      for (int64_t j = 0; j < c; ++j) {
        const uint32_t v = x[j] + a;
        x[j + deg] = v;
        o[j] = (int32_t)(v >> 1);
        a = b;
        b = d;
        d = v;
      }
    } else {
      uint32_t d = x[deg - 1];
      for (int64_t j = 0; j < c; ++j) {
        const uint32_t v = x[j] + d;
        x[j + deg] = v;
        o[j] = (int32_t)(v >> 1);
        d = v;
      }
    }
    memmove(x, x + c, sizeof(uint32_t) * (size_t)deg);
    done += c;
  }
  memcpy(win, w.data(), sizeof(uint32_t) * (size_t)deg);
}

// a * b mod the characteristic polynomial x^deg - x^(deg-sep) - 1 of the
// recurrence, coefficients mod 2^32 (x^d = x^(d-sep) + x^(d-deg) for d >= deg)
std::vector<uint32_t> polymul(const std::vector<uint32_t> &a, const std::vector<uint32_t> &b,
                              int deg, int sep) {
  std::vector<uint32_t> r((size_t)(2 * deg - 1), 0u);
  for (int i = 0; i < deg; ++i)
    for (int k = 0; k < deg; ++k) r[(size_t)(i + k)] += a[(size_t)i] * b[(size_t)k];
  for (int d = 2 * deg - 2; d >= deg; --d) {
    r[(size_t)(d - sep)] += r[(size_t)d];
    r[(size_t)(d - deg)] += r[(size_t)d];
  }
  r.resize((size_t)deg);
  return r;
}

// the window x_s .. x_{s+deg-1} from the window x_0 .. x_{deg-1}: with
// x^(s+i) = sum_j q_j x^j mod the characteristic polynomial, x_{s+i} = sum_j q_j x_j
void lfg_jump(const uint32_t *x0, int deg, int sep, int64_t s, uint32_t *win) {
  std::vector<uint32_t> q((size_t)deg, 0u), base((size_t)deg, 0u);
  q[0] = 1u;
  base[1] = 1u;                                  // the polynomial x
  for (int64_t e = s; e > 0; e >>= 1) {
    if (e & 1) q = polymul(q, base, deg, sep);
    base = polymul(base, base, deg, sep);
  }
  for (int i = 0; i < deg; ++i) {
    uint32_t v = 0u;
    for (int j = 0; j < deg; ++j) v += q[(size_t)j] * x0[j];
    win[i] = v;
    // q <- x q
    const uint32_t top = q[(size_t)(deg - 1)];
    for (int j = deg - 1; j > 0; --j) q[(size_t)j] = q[(size_t)(j - 1)];
    q[0] = top;
    q[(size_t)(deg - sep)] += top;
  }
}

// n values of the recurrence from the ring of a state buffer (header word
// first), advancing the ring and the header's position.  Long runs are split
// over host threads, each starting from its own window (lfg_jump).
void lfg_draw(char *state, int32_t *out, int64_t n) {
  int32_t hdr;
  memcpy(&hdr, state, sizeof hdr);
  const int type = hdr % MAX_TYPES, deg = DEG[type], sep = SEP[type];
  const int64_t rear = hdr / MAX_TYPES;
  std::vector<uint32_t> ring((size_t)deg);
  memcpy(ring.data(), state + sizeof(int32_t), sizeof(uint32_t) * (size_t)deg);
  // x_0 .. x_{deg-1}: the ring read from the slot the next value replaces
  const int f0 = (int)((rear + sep) % deg);
  std::vector<uint32_t> x0((size_t)deg);
  for (int i = 0; i < deg; ++i) x0[(size_t)i] = ring[(size_t)((f0 + i) % deg)];
  int T = 1;
  if (n >= ((int64_t)1 << 22)) T = std::max(1, std::min(omp_get_max_threads(), 32));
  const int64_t L = (n + T - 1) / T;
  std::vector<uint32_t> last(x0);
#pragma omp parallel for num_threads(T) schedule(static, 1)
  for (int t = 0; t < T; ++t) {
    const int64_t s = (int64_t)t * L, e = std::min(n, s + L);
    if (s >= e) continue;
    std::vector<uint32_t> win((size_t)deg);
    if (s == 0) win = x0;
    else lfg_jump(x0.data(), deg, sep, s, win.data());
    lfg_run(win.data(), deg, sep, out + s, e - s);
    if (e == n) last = win;
  }
  // the ring after n steps: slot (f0 + n + i) mod deg holds x_{n+i}
  const int fn = (int)((f0 + n) % deg);
  for (int i = 0; i < deg; ++i) ring[(size_t)((fn + i) % deg)] = last[(size_t)i];
  memcpy(state + sizeof(int32_t), ring.data(), sizeof(uint32_t) * (size_t)deg);
  const int32_t nh = (int32_t)(MAX_TYPES * ((rear + n) % deg) + type);
  memcpy(state, &nh, sizeof nh);
}

// whether state holds an additive state this code reads: type 1-4, rear in the ring
bool additive(const char *state) {
  int32_t hdr;
  memcpy(&hdr, state, sizeof hdr);
  if (hdr < 0) return false;
  const int type = hdr % MAX_TYPES;
  return type >= 1 && hdr / MAX_TYPES < DEG[type];
}

#if defined(__GLIBC__)
// The bulk path against rand() itself, on scratch states (the process's state
// is swapped out meanwhile and swapped back unchanged).
bool self_check() {
  alignas(8) char scratch[4 + 4 * 63] = {};
  alignas(8) char probe[128];
  const int32_t h3 = 3;                      // type 3, rear 0
  memcpy(scratch, &h3, sizeof h3);
  char *mine = setstate(scratch);            // the process's state, position saved
  if (!mine) return false;
  bool ok = initstate(12345u, probe, sizeof probe) != nullptr;   // type 3, seeded
  if (ok) {
    for (int i = 0; i < 5; ++i) (void)rand();
    char *p = setstate(scratch);               // probe's position saved into probe
    ok = p == probe && additive(probe);
    if (ok) {
      alignas(8) char copy[sizeof probe];
      memcpy(copy, probe, sizeof probe);
      int32_t bulk[1000];
      lfg_draw(copy, bulk, 1000);
      setstate(probe);
      for (int i = 0; i < 1000 && ok; ++i) ok = rand() == bulk[i];
      // the state left behind must continue the same way
      if (ok) {
        setstate(scratch);
        ok = memcmp(copy, probe, sizeof probe) == 0;
      }
    }
  }
  setstate(mine);
  return ok;
}
#endif

}  // namespace

// (declared in moc_internal.h)
int moc_libc_draws(int32_t *out, int64_t n) {
  if (n <= 0) return 0;
#if defined(__GLIBC__)
  static std::once_flag once;
  static bool bulk_ok = false;
  std::call_once(once, [] { bulk_ok = self_check(); });
  if (bulk_ok) {
    alignas(8) char scratch[4 + 4 * 63] = {};
    const int32_t h3 = 3;
    memcpy(scratch, &h3, sizeof h3);
    char *mine = setstate(scratch);
    if (mine && additive(mine)) {
      lfg_draw(mine, out, n);
      setstate(mine);
      return 1;
    }
    if (mine) setstate(mine);
  }
#endif
  for (int64_t k = 0; k < n; ++k) out[k] = rand();
  return 0;
}
