// The AO stage's per-sample random offsets, (float) rand() / RAND_MAX in the
// reference (lighter_int.hpp:271, drawn per sample at lighter.cpp:819), drawn
// in bulk. Each rand() call takes the C library's generator lock, so a
// million draws cost tens of milliseconds on one thread; here the values come
// from the generator's own recurrence without the lock:
//
// glibc's rand() is random() with the default state of type 3 (BSD
// random(3)): an additive feedback generator over 31 words,
//     r[f] += r[b];  output = r[f] >> 1;  f, b advance by one modulo 31,
// with the front index 3 ahead of the rear one. initstate() and setstate()
// switch the state array in use; on a switch the library records the rear
// index of the array it leaves in the word before the array (type + 5 * rear).
// rand_floats parks the generator on a scratch array, steps the parked state
// n times, writes it back (words and rear index) and switches back to it, so
// the values and the state after the call are those of n rand() calls.
// States of other types (a caller's initstate() with another size) take the
// rand() loop. The library is not told of another thread's rand() calls
// between the two switches; the reference draws from its bake thread too.
#include <cstdint>
#include <cstdlib>
#include <mutex>

#include "scene.hpp"

namespace lg {

namespace {
std::mutex g_rand_mu;
constexpr int kMaxTypes = 5, kType3 = 3, kDeg3 = 31, kSep3 = 3;
}  // namespace

void rand_floats(float* out, size_t n)
{
    std::lock_guard<std::mutex> lk(g_rand_mu);
#if defined(__GLIBC__)
    alignas(8) static char scratch[128];
    char* old = initstate(1u, scratch, sizeof(scratch));   // parks the process state, recording its rear index
    if (old) {
        int32_t* w = reinterpret_cast<int32_t*>(old);
        const int type = w[0] % kMaxTypes;
        if (type == kType3) {
            uint32_t* r = reinterpret_cast<uint32_t*>(w + 1);
            int b = w[0] / kMaxTypes;
            int f = (b + kSep3) % kDeg3;
            for (size_t i = 0; i < n; ++i) {
                r[f] += r[b];
                out[i] = (float) (int) (r[f] >> 1) / (float) RAND_MAX;
                if (++f == kDeg3) f = 0;
                if (++b == kDeg3) b = 0;
            }
            w[0] = kMaxTypes * b + type;
            setstate(old);
            return;
        }
        setstate(old);   // another state type: draw through rand()
    }
#endif
    for (size_t i = 0; i < n; ++i) out[i] = (float) rand() / (float) RAND_MAX;
}

}  // namespace lg

extern "C" LTRAPI void ltrdbg_DrawRandFloats(float* out, u32 n)
{
    if (out) lg::rand_floats(out, n);
}
