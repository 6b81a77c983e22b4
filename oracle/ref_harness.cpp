/*
 * ref_harness.cpp — TEST INFRASTRUCTURE.  Compiles the reference's own
 * header-only routines straight from its source tree (never copied here):
 *   halmd/mdsim/sorts/hilbert_kernel.hpp   (Hilbert map, host instantiation)
 *   halmd/numeric/mp/dsfun.hpp             (dsadd / dssub / dsmul)
 * and evaluates them on inputs read from stdin, so that tests/golden/ can
 * pin the oracle's restatements (oracle/oracle.cpp) against the reference.
 *
 * stdin protocol (text):
 *   hilbert <depth> <n>  then n lines "x y z" (unit-cube coordinates, float)
 *       -> n lines with the key
 *   dsfun <op> <n>       then n lines "a0 a1 b0 b1" (hex float bits)
 *       -> n lines "c0 c1" (hex float bits); op = add | sub | mul
 */
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

namespace shim {
struct vec3 {
    typedef float value_type;
    enum { static_size = 3 };
    float v[3];
    vec3() {}
    explicit vec3(float s) { v[0] = v[1] = v[2] = s; }
    float& operator[](int i) { return v[i]; }
    float const& operator[](int i) const { return v[i]; }
    vec3& operator*=(float s) { for (int i = 0; i < 3; ++i) v[i] *= s; return *this; }
    vec3& operator-=(vec3 const& o) { for (int i = 0; i < 3; ++i) v[i] -= o.v[i]; return *this; }
};
inline vec3 operator-(vec3 a, vec3 const& b) { for (int i = 0; i < 3; ++i) a.v[i] -= b.v[i]; return a; }
inline vec3 operator+(vec3 a, vec3 const& b) { for (int i = 0; i < 3; ++i) a.v[i] += b.v[i]; return a; }
inline vec3 operator*(vec3 a, float s) { for (int i = 0; i < 3; ++i) a.v[i] *= s; return a; }
inline vec3 operator/(vec3 a, float s) { for (int i = 0; i < 3; ++i) a.v[i] /= s; return a; }
inline vec3 floor(vec3 a) { for (int i = 0; i < 3; ++i) a.v[i] = std::floor(a.v[i]); return a; }
} // namespace shim

#include <halmd/mdsim/sorts/hilbert_kernel.hpp>
#include <halmd/numeric/mp/dsfun.hpp>

static float from_hex(unsigned u) { float f; std::memcpy(&f, &u, 4); return f; }
static unsigned to_hex(float f) { unsigned u; std::memcpy(&u, &f, 4); return u; }

int main()
{
    char cmd[32];
    while (std::scanf("%31s", cmd) == 1) {
        if (std::string(cmd) == "hilbert") {
            unsigned depth; int n;
            if (std::scanf("%u %d", &depth, &n) != 2) return 1;
            for (int i = 0; i < n; ++i) {
                shim::vec3 r;
                if (std::scanf("%f %f %f", &r[0], &r[1], &r[2]) != 3) return 1;
                std::printf("%u\n", halmd::mdsim::sorts::hilbert_kernel::map(r, depth));
            }
        } else if (std::string(cmd) == "dsfun") {
            char op[8]; int n;
            if (std::scanf("%7s %d", op, &n) != 2) return 1;
            for (int i = 0; i < n; ++i) {
                unsigned a0, a1, b0, b1;
                if (std::scanf("%x %x %x %x", &a0, &a1, &b0, &b1) != 4) return 1;
                float c0, c1;
                using namespace halmd::detail::numeric::mp;
                if (std::string(op) == "add") dsadd(c0, c1, from_hex(a0), from_hex(a1), from_hex(b0), from_hex(b1));
                else if (std::string(op) == "sub") dssub(c0, c1, from_hex(a0), from_hex(a1), from_hex(b0), from_hex(b1));
                else dsmul(c0, c1, from_hex(a0), from_hex(a1), from_hex(b0), from_hex(b1));
                std::printf("%08x %08x\n", to_hex(c0), to_hex(c1));
            }
        } else {
            return 2;
        }
    }
    return 0;
}
