/*
 * port.cpp - CPU restatement of the reference's PM / P3M force-and-step path.
 * TEST INFRASTRUCTURE ONLY ("the oracle"): tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline legs call it as the reference results or as the timed CPU baseline; the product
 * (particlesimulation_gb300/, include/) never links it.
 *
 * Everything is templated on the scalar type T.  T = float repeats the reference's FP32
 * arithmetic operation by operation (so it tracks the reference to rounding level and is
 * the CPU baseline when the reference itself cannot be compiled, e.g. on a machine without
 * its sources); T = double is the FP64 oracle.  It is pinned against the reference compiled
 * from its own sources (oracle/_ref, see oracle/Makefile) by tests/test_oracle_pin.py and
 * against golden fixtures generated from it (tests/golden/).
 *
 * Reference functions restated here (paths within the reference project):
 *   units           include/unitConversions.h:8-50
 *   Green functions source/greensFunctions.cpp:8-221
 *   spreadMass      source/pmMethod.cpp:187-277   (TSCAssignmentFunc 187-198)
 *   interpolation   source/pmMethod.cpp:279-338, updateAccelerations 384-390
 *   Fourier pot.    source/pmMethod.cpp:340-350
 *   FD field        source/pmMethod.cpp:352-382, Grid::getPotential source/grid.cpp:66-68
 *   FFT             FFTAdapter::fft / ifft (include/kissFFTAdapter.h:16-29): forward
 *                   unnormalised e^{-i}, inverse e^{+i} divided by the element count.
 *                   The transform itself is our own radix-2 / direct DFT, not kissfft.
 *   leapfrog        source/leapfrog.cpp:5-24
 *   PM run loop     source/pmMethod.cpp:62-135
 *   SR force        source/p3mMethod.cpp:194-294
 *   pair pass       source/p3mMethod.cpp:168-192, 247-273, 296-322
 *   correctAcc      source/p3mMethod.cpp:50-57
 *   P3M run loop    source/p3mMethod.cpp:59-166
 *   chaining mesh   source/chainingMesh.cpp:6-84
 *   direct sum      source/ppMethod.cpp:23-36 (in double, targets x all sources)
 *
 * Deliberate differences (documented, test-visible):
 *   - mesh indices of deposits and field reads are wrapped periodically; the reference
 *     leaves them unwrapped (undefined behaviour for particles within a stencil of the mesh
 *     edge), so results agree wherever the reference is defined.
 *   - double only: the optimal Green's function is set to 0 at the 7 non-zero modes whose
 *     components are all 0 or N/2, where the finite-difference operator vanishes and the
 *     reference divides float rounding noise by rounding noise.  The force is blind to
 *     those modes (the FD gradient annihilates them).
 */
#include <algorithm>
#include <array>
#include <atomic>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <numbers>
#include <thread>
#include <type_traits>
#include <vector>

#include "oracle_api.h"

namespace {

template <typename T>
struct V3 {
  T x{}, y{}, z{};
};
template <typename T>
inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename T>
inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename T>
inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <typename T>
inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <typename T>
inline V3<T>& operator+=(V3<T>& a, V3<T> b) {
  a.x += b.x;
  a.y += b.y;
  a.z += b.z;
  return a;
}
template <typename T>
inline T mag2(V3<T> a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
template <typename T>
inline T mag(V3<T> a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

void parallel_for(int n, int nthreads, const std::function<void(int, int)>& body) {
  if (nthreads <= 1 || n < 2) {
    body(0, n);
    return;
  }
  std::vector<std::thread> th;
  int chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    int b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back(body, b, e);
  }
  for (auto& x : th) x.join();
}

/* ------------------------------------------------------------------ FFT ---- */
template <typename T>
struct FFT1 {
  int n = 0;
  bool pow2 = false;
  std::vector<std::complex<T>> tw;  // e^{-2 pi i k / n}, computed in double
  std::vector<int> rev;
  explicit FFT1(int n_) : n(n_) {
    pow2 = n > 0 && (n & (n - 1)) == 0;
    tw.resize(n);
    for (int k = 0; k < n; ++k) {
      double a = -2.0 * std::numbers::pi * double(k) / double(n);
      tw[k] = std::complex<T>(T(std::cos(a)), T(std::sin(a)));
    }
    if (pow2) {
      rev.resize(n);
      int lg = 0;
      while ((1 << lg) < n) ++lg;
      for (int i = 0; i < n; ++i) {
        int r = 0;
        for (int b = 0; b < lg; ++b)
          if (i & (1 << b)) r |= 1 << (lg - 1 - b);
        rev[i] = r;
      }
    }
  }
  // in-place transform of a contiguous line; sign -1 forward, +1 inverse (unnormalised)
  void run(std::complex<T>* a, bool inverse, std::vector<std::complex<T>>& tmp) const {
    if (n == 1) return;
    if (pow2) {
      for (int i = 0; i < n; ++i)
        if (i < rev[i]) std::swap(a[i], a[rev[i]]);
      for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1, step = n / len;
        for (int s = 0; s < n; s += len) {
          for (int j = 0; j < half; ++j) {
            std::complex<T> w = tw[j * step];
            if (inverse) w = std::conj(w);
            std::complex<T> u = a[s + j], v = a[s + j + half] * w;
            a[s + j] = u + v;
            a[s + j + half] = u - v;
          }
        }
      }
    } else {
      tmp.assign(a, a + n);
      for (int k = 0; k < n; ++k) {
        std::complex<T> acc(0, 0);
        for (int j = 0; j < n; ++j) {
          std::complex<T> w = tw[(int64_t(j) * k) % n];
          if (inverse) w = std::conj(w);
          acc += tmp[j] * w;
        }
        a[k] = acc;
      }
    }
  }
};

template <typename T>
struct FFT3 {
  int nx, ny, nz;
  FFT1<T> fx, fy, fz;
  FFT3(int x, int y, int z) : nx(x), ny(y), nz(z), fx(x), fy(y), fz(z) {}
  void run(std::vector<std::complex<T>>& d, bool inverse, int nthreads) const {
    // x lines (contiguous)
    parallel_for(ny * nz, nthreads, [&](int b, int e) {
      std::vector<std::complex<T>> tmp;
      for (int r = b; r < e; ++r) fx.run(d.data() + size_t(r) * nx, inverse, tmp);
    });
    parallel_for(nx * nz, nthreads, [&](int b, int e) {
      std::vector<std::complex<T>> line(ny), tmp;
      for (int r = b; r < e; ++r) {
        int x = r % nx, z = r / nx;
        for (int y = 0; y < ny; ++y) line[y] = d[(size_t(z) * ny + y) * nx + x];
        fy.run(line.data(), inverse, tmp);
        for (int y = 0; y < ny; ++y) d[(size_t(z) * ny + y) * nx + x] = line[y];
      }
    });
    parallel_for(nx * ny, nthreads, [&](int b, int e) {
      std::vector<std::complex<T>> line(nz), tmp;
      for (int r = b; r < e; ++r) {
        for (int z = 0; z < nz; ++z) line[z] = d[size_t(z) * nx * ny + r];
        fz.run(line.data(), inverse, tmp);
        for (int z = 0; z < nz; ++z) d[size_t(z) * nx * ny + r] = line[z];
      }
    });
    if (inverse) {
      T len = static_cast<T>(nx * ny * nz);
      for (auto& x : d) x /= len;
    }
  }
};

/* ------------------------------------------------------- Green functions ---- */
template <typename T>
constexpr T PI = std::numbers::pi_v<T>;

template <typename T>
T sinc(T x) { return x == 0 ? T(1) : std::sin(x) / x; }
template <typename T>
T powT(T x, T e) { return std::pow(x, e); }

template <typename T>
T assignFourier(int is, const T k[3]) {  // TSC/CIC/NGPFourier (greensFunctions.cpp:15-40)
  T prod = 1;
  for (int i = 0; i < 3; i++) {
    if (is == 2) prod *= powT(sinc(k[i] / 2), T(3));
    else if (is == 1) prod *= powT(sinc(k[i] / 2), T(2));
    else prod *= sinc(k[i] / 2);
  }
  return prod;
}
template <typename T>
T aliasSum(int is, const T k[3]) {  // *AliasSum (greensFunctions.cpp:102-120)
  if (is == 2) {
    T sum = 1;
    for (int i = 0; i < 3; i++)
      sum *= (1 - powT(std::sin(k[i] / 2), T(2)) + T(2) / 15 * powT(std::sin(k[i] / 2), T(4)));
    return sum;
  }
  if (is == 1) {
    T sum = 1;
    for (int i = 0; i < 3; i++) sum *= (1 + 2 * powT(std::cos(k[i] / 2), T(2)));
    return (T(1) / 27) * sum;
  }
  return 1;
}
template <typename T>
T shapeFourier(int cs, T k, T a) {  // S1Fourier / S2Fourier (greensFunctions.cpp:42-50)
  T u = k * a / 2;
  if (cs == 0) return -3 / powT(u, T(3)) * (u * std::cos(u) - std::sin(u));
  return 12 / powT(u, T(4)) * (2 - 2 * std::cos(u) - u * std::sin(u));
}

template <typename T>
T greenOptimal(int is, int kx, int ky, int kz, int nx, int ny, int nz, T a, int cs, int fds) {
  using C = std::complex<T>;
  if (kx == 0 && ky == 0 && kz == 0) return 0;
  if constexpr (std::is_same_v<T, double>) {
    // all components 0 or N/2: the FD operator D(k) is identically zero (see header)
    auto edge = [](int k, int n) { return k == 0 || 2 * k == n; };
    if (edge(kx, nx) && edge(ky, ny) && edge(kz, nz)) return 0;
  }
  T k[3] = {2 * PI<T> * T(kx) / nx, 2 * PI<T> * T(ky) / ny, 2 * PI<T> * T(kz) / nz};
  T denomSum = aliasSum<T>(is, k);
  const C I(0, 1);
  C D[3];
  if (fds == 0) {
    for (int i = 0; i < 3; i++) D[i] = I * std::sin(k[i]);
  } else {
    T alpha = T(4) / 3;
    for (int i = 0; i < 3; i++)
      D[i] = I * alpha * std::sin(k[i]) + I * (1 - alpha) * std::sin(2 * k[i]) / T(2);
  }
  auto dot = [](const C* a, const C* b) {
    C d(0, 0);
    for (int i = 0; i < 3; i++) d += a[i] * C(b[i].real(), -1 * b[i].imag());
    return d;
  };
  T DNormSquared = dot(D, D).real();
  C num[3] = {C(0, 0), C(0, 0), C(0, 0)};
  const int limit = 2;
  for (int n1 = -limit; n1 <= limit; n1++)
    for (int n2 = -limit; n2 <= limit; n2++)
      for (int n3 = -limit; n3 <= limit; n3++) {
        T kn[3] = {k[0] + 2 * PI<T> * n1, k[1] + 2 * PI<T> * n2, k[2] + 2 * PI<T> * n3};
        T uSquared = powT(assignFourier<T>(is, kn), T(2));
        T kLength = std::sqrt(kn[0] * kn[0] + kn[1] * kn[1] + kn[2] * kn[2]);
        T s = shapeFourier<T>(cs, kLength, a);
        T sSquared = powT(s, T(2));
        for (int i = 0; i < 3; i++) {
          C R = -I * kn[i] * sSquared / (kLength * kLength);
          num[i] += uSquared * R;
        }
      }
  C numerator = dot(D, num);
  T denominator = DNormSquared * denomSum * denomSum;
  return (numerator / denominator).real();
}

template <typename T>
T greenValue(const orc_pm_params* p, T diameterCode, int kx, int ky, int kz) {
  int nx = p->nx, ny = p->ny, nz = p->nz;
  if (p->gf == 0) {  // GreenDiscreteLaplacian (greensFunctions.cpp:191-200)
    if (kx == 0 && ky == 0 && kz == 0) return 0;
    T sx = std::sin(PI<T> * kx / nx), sy = std::sin(PI<T> * ky / ny), sz = std::sin(PI<T> * kz / nz);
    return T(-0.25) / (sx * sx + sy * sy + sz * sz);
  }
  if (p->gf == 3) {  // GreenPoorMan (greensFunctions.cpp:202-221)
    if (kx == 0 && ky == 0 && kz == 0) return 0;
    int ki = (kx <= nx / 2) ? kx : kx - nx;
    int kj = (ky <= ny / 2) ? ky : ky - ny;
    int kk = (kz <= nz / 2) ? kz : kz - nz;
    T fx = 2 * PI<T> * ki / nx, fy = 2 * PI<T> * kj / ny, fz = 2 * PI<T> * kk / nz;
    return T(-1) / (fx * fx + fy * fy + fz * fz);
  }
  int cs = p->gf == 1 ? 0 : 1;
  // is = 3 (centred TSC, a deviation from the reference) has TSC's assignment function
  return greenOptimal<T>(p->is == 3 ? 2 : p->is, kx, ky, kz, nx, ny, nz, diameterCode, cs, p->fds);
}

/* ------------------------------------------------------------------- PM ---- */
template <typename T>
T tscW(T x, int t) {  // PMMethod::TSCAssignmentFunc (pmMethod.cpp:187-198)
  if (t == 1) return (T(0.5) + x) * (T(0.5) + x);
  if (t == 0) return T(1.5) - 2 * x * x;
  if (t == -1) return (T(0.5) - x) * (T(0.5) - x);
  return 0;
}

inline int wrap(int a, int b) { return (a % b + b) % b; }

template <typename T>
struct PM {
  orc_pm_params p;
  int N, nx, ny, nz;
  size_t L;
  T H, DT, G, diam;
  std::vector<V3<T>> x, v, a;
  std::vector<T> m;
  std::vector<std::complex<T>> dens, potF, pot;
  std::vector<T> green;
  std::vector<V3<T>> field;
  FFT3<T> fft;
  int nthreads;

  PM(const orc_pm_params* pp, int n, const float* state, const float* masses, int nth)
      : p(*pp), N(n), nx(pp->nx), ny(pp->ny), nz(pp->nz),
        L(size_t(pp->nx) * pp->ny * pp->nz), H(pp->H), DT(pp->DT), G(pp->G),
        fft(pp->nx, pp->ny, pp->nz), nthreads(nth) {
    diam = T(pp->diameter) / H;  // lengthToCodeUnits
    x.resize(n);
    v.resize(n);
    a.resize(n);
    m.resize(n);
    for (int i = 0; i < n; ++i) {
      x[i] = {T(state[3 * i]), T(state[3 * i + 1]), T(state[3 * i + 2])};
      v[i] = {T(state[3 * (n + i)]), T(state[3 * (n + i) + 1]), T(state[3 * (n + i) + 2])};
      m[i] = T(masses[i]);
    }
    dens.assign(L, 0);
    potF.assign(L, 0);
    pot.assign(L, 0);
    green.assign(L, 0);
    field.assign(L, V3<T>{});
  }
  size_t idx(int i, int j, int k) const {
    return size_t(wrap(i, nx)) + size_t(wrap(j, ny)) * nx + size_t(wrap(k, nz)) * nx * ny;
  }
  // stateToCodeUnits + massToCodeUnits (unitConversions.h:8-50)
  void toCode() {
    for (int i = 0; i < N; ++i) {
      x[i] = x[i] / H;
      v[i] = (DT * v[i]) / H;
      m[i] = DT * DT * 4 * PI<T> * G / (H * H * H) * m[i];
    }
  }
  void statesToOriginal() {
    for (int i = 0; i < N; ++i) {
      x[i] = H * x[i];
      v[i] = (H * v[i]) / DT;
    }
  }
  void statesToCode() {
    for (int i = 0; i < N; ++i) {
      x[i] = x[i] / H;
      v[i] = (DT * v[i]) / H;
    }
  }
  void initGreen() {
    parallel_for(int(L), nthreads, [&](int b, int e) {
      for (int id = b; id < e; ++id) {
        int kx = id % nx, ky = (id / nx) % ny, kz = id / (nx * ny);
        green[id] = greenValue<T>(&p, diam, kx, ky, kz);
      }
    });
  }
  // TSC's centre cell.  The reference (is = 2) centres the 3-point stencil on the cell below
  // the particle (int(x), offsets in [0, 1): pmMethod.cpp:250-270, 312-331), so its weights
  // (TSCAssignmentFunc, pmMethod.cpp:187-198) jump where x crosses an integer and go negative
  // above sqrt(3)/2.  is = 3 (a deviation, not in the reference) centres it on the nearest
  // mesh point, offsets in [-1/2, 1/2]: the standard TSC of Hockney & Eastwood.
  void tscBase(const V3<T>& q, int& ix, int& iy, int& iz) const {
    if (p.is == 3) {
      ix = (int)std::floor(q.x + T(0.5));
      iy = (int)std::floor(q.y + T(0.5));
      iz = (int)std::floor(q.z + T(0.5));
    } else {
      ix = (int)q.x;
      iy = (int)q.y;
      iz = (int)q.z;
    }
  }
  void spreadMass() {
    std::fill(dens.begin(), dens.end(), std::complex<T>(0, 0));
    for (int i = 0; i < N; ++i) {
      const V3<T> q = x[i];
      if (p.is == 0) {
        int ix = (int)std::round(q.x), iy = (int)std::round(q.y), iz = (int)std::round(q.z);
        dens[idx(ix, iy, iz)] += m[i];
      } else if (p.is == 1) {
        int ix = (int)q.x, iy = (int)q.y, iz = (int)q.z;
        T d = m[i];
        T dx = q.x - ix, dy = q.y - iy, dz = q.z - iz;
        T tx = 1 - dx, ty = 1 - dy, tz = 1 - dz;
        dens[idx(ix, iy, iz)] += d * tx * ty * tz;
        dens[idx(ix + 1, iy, iz)] += d * dx * ty * tz;
        dens[idx(ix, iy + 1, iz)] += d * tx * dy * tz;
        dens[idx(ix, iy, iz + 1)] += d * tx * ty * dz;
        dens[idx(ix + 1, iy + 1, iz)] += d * dx * dy * tz;
        dens[idx(ix + 1, iy, iz + 1)] += d * dx * ty * dz;
        dens[idx(ix, iy + 1, iz + 1)] += d * tx * dy * dz;
        dens[idx(ix + 1, iy + 1, iz + 1)] += d * dx * dy * dz;
      } else {
        int ix, iy, iz;
        tscBase(q, ix, iy, iz);
        T d = m[i];
        T dx = q.x - ix, dy = q.y - iy, dz = q.z - iz;
        for (int t1 = -1; t1 <= 1; ++t1) {
          T T1 = (d / 8) * tscW(dx, t1);
          for (int t2 = -1; t2 <= 1; ++t2) {
            T T2 = T1 * tscW(dy, t2);
            for (int t3 = -1; t3 <= 1; ++t3) {
              T T3 = T2 * tscW(dz, t3);
              dens[idx(ix + t1, iy + t2, iz + t3)] += T3;
            }
          }
        }
      }
    }
  }
  T phi(int i, int j, int k) const { return pot[idx(i, j, k)].real(); }
  void findField() {
    parallel_for(int(L), nthreads, [&](int b, int e) {
      for (int id = b; id < e; ++id) {
        int i = id % nx, j = (id / nx) % ny, k = id / (nx * ny);
        V3<T> f;
        if (p.fds == 0) {
          f.x = T(-0.5) * (phi(i + 1, j, k) - phi(i - 1, j, k));
          f.y = T(-0.5) * (phi(i, j + 1, k) - phi(i, j - 1, k));
          f.z = T(-0.5) * (phi(i, j, k + 1) - phi(i, j, k - 1));
        } else {
          T c = T(-1.0) / 12;
          f.x = c * (-phi(i + 2, j, k) + 8 * phi(i + 1, j, k) - 8 * phi(i - 1, j, k) + phi(i - 2, j, k));
          f.y = c * (-phi(i, j + 2, k) + 8 * phi(i, j + 1, k) - 8 * phi(i, j - 1, k) + phi(i, j - 2, k));
          f.z = c * (-phi(i, j, k + 2) + 8 * phi(i, j, k + 1) - 8 * phi(i, j, k - 1) + phi(i, j, k - 2));
        }
        field[id] = f;
      }
    });
  }
  V3<T> fieldAt(int i, int j, int k) const { return field[idx(i, j, k)]; }
  V3<T> interpolate(V3<T> q) const {
    if (p.is == 0) {
      return fieldAt((int)std::round(q.x), (int)std::round(q.y), (int)std::round(q.z));
    }
    int xi = (int)q.x, yi = (int)q.y, zi = (int)q.z;
    if (p.is >= 2) tscBase(q, xi, yi, zi);
    T dx = q.x - xi, dy = q.y - yi, dz = q.z - zi;
    if (p.is == 1) {
      T tx = 1 - dx, ty = 1 - dy, tz = 1 - dz;
      return tx * ty * tz * fieldAt(xi, yi, zi) + dx * ty * tz * fieldAt(xi + 1, yi, zi) +
             tx * dy * tz * fieldAt(xi, yi + 1, zi) + tx * ty * dz * fieldAt(xi, yi, zi + 1) +
             dx * dy * tz * fieldAt(xi + 1, yi + 1, zi) + dx * ty * dz * fieldAt(xi + 1, yi, zi + 1) +
             tx * dy * dz * fieldAt(xi, yi + 1, zi + 1) + dx * dy * dz * fieldAt(xi + 1, yi + 1, zi + 1);
    }
    V3<T> r;
    for (int t1 = -1; t1 <= 1; ++t1) {
      T T1 = tscW(dx, t1);
      for (int t2 = -1; t2 <= 1; ++t2) {
        T T2 = T1 * tscW(dy, t2);
        for (int t3 = -1; t3 <= 1; ++t3) {
          T T3 = T2 * tscW(dz, t3);
          r += (T(0.125) * T3) * fieldAt(xi + t1, yi + t2, zi + t3);
        }
      }
    }
    return r;
  }
  V3<T> external(V3<T> q) const {  // sphRadDecrField at H*x, converted to code units
    if (p.ext_kind != 1) return {};
    V3<T> pos = H * q;
    V3<T> c{T(p.ext_cx), T(p.ext_cy), T(p.ext_cz)};
    T R = p.ext_R, M = p.ext_M, Gx = p.ext_G;
    T r = mag(pos - c);
    V3<T> dir = (pos - c) / r;
    T g = r > R ? -Gx * M / (r * r) : -(Gx * M / powT(R, T(3))) * r * (4 - 3 * r / R);
    V3<T> f = g * dir;
    return (DT * DT * f) / H;
  }
  std::vector<T> rhoReal;  // density of the last step (the FFT below overwrites dens)
  void step() {  // pmMethodStep (pmMethod.cpp:137-144)
    spreadMass();
    rhoReal.resize(L);
    for (size_t id = 0; id < L; ++id) rhoReal[id] = dens[id].real();
    fft.run(dens, false, nthreads);
    potF = dens;
    for (size_t id = 0; id < L; ++id) potF[id] = dens[id] * std::complex<T>(green[id], 0);
    potF[0] = 0;
    pot = potF;
    fft.run(pot, true, nthreads);
    findField();
    parallel_for(N, nthreads, [&](int b, int e) {
      for (int i = b; i < e; ++i) a[i] = interpolate(x[i]) + external(x[i]);
    });
  }
  bool escaped() const {  // escapedComputationalBox on original-unit positions
    for (int i = 0; i < N; ++i) {
      const V3<T>& q = x[i];
      if (!(q.x >= 0 && q.x <= p.box_x && q.y >= 0 && q.y <= p.box_y && q.z >= 0 && q.z <= p.box_z))
        return true;
    }
    return false;
  }
};

/* ------------------------------------------------------------------ P3M ---- */
template <typename T>
struct ChainMesh {  // ChainingMesh (chainingMesh.cpp:6-84): linked lists over a node pool
  int Mx, My, Mz, size;
  T HCx, HCy, HCz;
  std::vector<int> hoc, next;
  ChainMesh(const orc_p3m_params* q, T H, int N) {
    Mx = int(q->comp_x / q->cutoff);
    My = int(q->comp_y / q->cutoff);
    Mz = int(q->comp_z / q->cutoff);
    HCx = T(q->comp_x / Mx) / H;  // lengthToCodeUnits(compBox/M, H); compBox/M in float
    HCy = T(q->comp_y / My) / H;
    HCz = T(q->comp_z / Mz) / H;
    size = Mx * My * Mz;
    hoc.assign(size, -1);
    next.assign(N, -1);
  }
  int flat(int x, int y, int z) const {
    if (x < 0 || y < 0 || z < 0 || x >= Mx || y >= My || z >= Mz) return -1;
    return x + y * Mx + z * Mx * My;
  }
  int cellOf(const V3<T>& q) const { return flat(int(q.x / HCx), int(q.y / HCy), int(q.z / HCz)); }
  void fill(const std::vector<V3<T>>& x, bool ysort) {
    std::fill(hoc.begin(), hoc.end(), -1);
    for (int i = 0; i < int(x.size()); ++i) {
      int c = cellOf(x[i]);
      if (c < 0) continue;  // the reference indexes hoc[-1] here (undefined)
      int head = hoc[c];
      if (!ysort) {
        next[i] = head;
        hoc[c] = i;
        continue;
      }
      if (head < 0 || x[head].y > x[i].y) {
        next[i] = head;
        hoc[c] = i;
        continue;
      }
      for (int node = head; node >= 0; node = next[node]) {
        if (next[node] < 0 || x[next[node]].y > x[i].y) {
          next[i] = next[node];
          next[node] = i;
          break;
        }
      }
    }
  }
  // The lists fill(x, true) builds (ascending y, ties in index order), by a stable sort of each
  // cell's particles instead of the reference's insertion sort (same order, O(n log n)); also
  // kept as arrays (cellOrder[cellStart[c] .. cellStart[c+1])).
  void fillSorted(const std::vector<V3<T>>& x) {
    std::fill(hoc.begin(), hoc.end(), -1);
    std::vector<std::vector<int>> cells(size);
    for (int i = 0; i < int(x.size()); ++i) {
      int c = cellOf(x[i]);
      if (c >= 0) cells[c].push_back(i);
    }
    cellStart.assign(size + 1, 0);
    cellOrder.clear();
    for (int c = 0; c < size; ++c) {
      auto& v = cells[c];
      std::stable_sort(v.begin(), v.end(), [&](int a, int b) { return x[a].y < x[b].y; });
      for (int k = int(v.size()) - 1; k >= 0; --k) {
        next[v[k]] = hoc[c];
        hoc[c] = v[k];
      }
      cellOrder.insert(cellOrder.end(), v.begin(), v.end());
      cellStart[c + 1] = int(cellOrder.size());
    }
  }
  std::vector<int> cellStart, cellOrder;
  void neighbors(int cell, int out[14]) const {
    int cx = cell % Mx, cy = (cell / Mx) % My, cz = cell / (Mx * My);
    int i = 0;
    for (int t = -1; t <= 1; ++t)
      for (int s = -1; s <= 1; ++s) out[i++] = flat(cx + t, cy - 1, cz + s);
    for (int s = -1; s <= 1; ++s) out[i++] = flat(cx + s, cy, cz - 1);
    out[12] = flat(cx - 1, cy, cz);
    out[13] = cell;
  }
};

template <typename T>
struct P3M {
  orc_p3m_params q;
  PM<T>& pm;
  ChainMesh<T> cm;
  T re, diam, eps, delta2;
  std::vector<T> table;
  std::vector<V3<T>> sr;                 // shortRangeForce
  std::vector<std::array<V3<T>, 13>> slot;  // shortRangeFromNeighbor
  int nthreads;

  P3M(const orc_p3m_params* qq, PM<T>& p, int nth)
      : q(*qq), pm(p), cm(qq, T(p.p.H), p.N), nthreads(nth) {
    re = T(q.cutoff) / T(p.p.H);
    diam = T(q.diameter) / T(p.p.H);
    eps = T(q.softening) / T(p.p.H);
    delta2 = re * re / (500 - 1);
    if (q.use_table) initTable();
    sr.resize(p.N);
    slot.resize(p.N);
  }
  T refS1(T r) const {
    const T a = diam, G = 1 / (4 * PI<T>);
    if (r >= a) return G / (r * r);
    return G / (a * a) * (8 * r / a - 9 * r * r / (a * a) + 2 * powT(r / a, T(4)));
  }
  T refS2(T r) const {
    const T a = diam, G = 1 / (4 * PI<T>);
    const T u = 2 * r / a;
    if (u <= 1)
      return G / (35 * powT(a, T(2))) *
             (224 * u - 224 * powT(u, T(3)) + 70 * powT(u, T(4)) + 48 * powT(u, T(5)) - 21 * powT(u, T(6)));
    if (u <= 2)
      return G / (35 * powT(a, T(2))) *
             (12 / powT(u, T(2)) - 224 + 896 * u - 840 * powT(u, T(2)) + 224 * powT(u, T(3)) +
              70 * powT(u, T(4)) - 48 * powT(u, T(5)) + 7 * powT(u, T(6)));
    return G / (r * r);
  }
  void initTable() {
    table.clear();
    for (int i = 0; i < 500; ++i) {
      T rSquared = i * delta2;
      T r = std::sqrt(rSquared);
      T R = q.cloud_shape == 0 ? -refS1(r) : -refS2(r);
      T G = 1 / (4 * PI<T>);
      T totalForce = -G / (r * r + eps * eps);
      table.push_back(r == 0 ? T(0) : (totalForce - R) / std::sqrt(r * r + eps * eps));
    }
  }
  V3<T> srForce(V3<T> rij, T mi, T mj) const {
    if (!q.use_table) {
      T len = mag(rij);
      V3<T> dir = rij / len;
      T G = 1 / (4 * PI<T>);
      T R = q.cloud_shape == 0 ? refS1(len) : refS2(len);
      V3<T> Rij = (-mi * mj * R) * dir;
      V3<T> tot = (-G * mi * mj / (len * len + eps * eps)) * dir;
      return tot - Rij;
    }
    T ksi = mag2(rij) / delta2;
    int t = int(ksi);
    if (t > 498) t = 498;  // the reference would read one past the table here
    T F = mi * mj * (table[t] + (ksi - t) * (table[t + 1] - table[t]));
    return F * rij;
  }
  int pairStride = 1;  // timing samples: only every pairStride-th particle (by index) is an i
  // Oracle runs (not the timed CPU baseline): y-sorted lists built by the equivalent stable sort,
  // each j walk starting at the first particle with y >= y_i - re (the ones before it fail the
  // cutoff test, as the reference's own early break assumes for the ones after the window), and
  // cells taken by threads from a shared counter.  The pairs, their order per particle and every
  // accumulator's writer are the reference's (sr[i] is written by i's cell only, slot[j][s] by
  // the one cell whose neighbour s is j's cell), so the results are the same.
  bool fast = false;
  std::atomic<int> nextCell{0};
  void fastJob() {
    const auto& x = pm.x;
    const auto& m = pm.m;
    int nb[14];
    for (int c = nextCell.fetch_add(1); c < cm.size; c = nextCell.fetch_add(1)) {
      cm.neighbors(c, nb);
      for (int s = 0; s < 14; ++s) {
        const int cn = nb[s];
        if (cn < 0) continue;
        const int* jb = cm.cellOrder.data() + cm.cellStart[cn];
        const int* je = cm.cellOrder.data() + cm.cellStart[cn + 1];
        for (int k = cm.cellStart[c]; k < cm.cellStart[c + 1]; ++k) {
          const int i = cm.cellOrder[k];
          const T ylo = x[i].y - re;
          const int* j0 = std::lower_bound(jb, je, ylo, [&](int j, T v) { return x[j].y < v; });
          for (const int* pj = j0; pj < je; ++pj) {
            const int j = *pj;
            if (x[j].y - x[i].y > re) break;
            if (i == j) continue;
            V3<T> rij = x[i] - x[j];
            if (mag2(rij) >= re * re) continue;
            V3<T> f = srForce(rij, m[i], m[j]);
            sr[i] += f;
            if (cn != c) slot[j][s] += T(-1) * f;
          }
        }
      }
    }
  }
  void threadJob(int tid, int threads) {
    const auto& x = pm.x;
    const auto& m = pm.m;
    int nb[14];
    for (int c = tid; c < cm.size; c += threads) {
      cm.neighbors(c, nb);
      for (int s = 0; s < 14; ++s) {
        int cn = nb[s];
        if (cn < 0) continue;
        for (int i = cm.hoc[c]; i >= 0; i = cm.next[i]) {
          // timing samples: every pairStride-th particle by index (unrelated to its place in
          // the y-sorted list, whose early break makes low-y particles cheaper)
          if (pairStride > 1 && i % pairStride) continue;
          for (int j = cm.hoc[cn]; j >= 0; j = cm.next[j]) {
            if (q.y_sorting && x[j].y - x[i].y > re) break;
            if (i == j) continue;
            V3<T> rij = x[i] - x[j];
            if (mag2(rij) >= re * re) continue;
            V3<T> f = srForce(rij, m[i], m[j]);
            sr[i] += f;
            if (cn != c) slot[j][s] += T(-1) * f;
          }
        }
      }
    }
  }
  void shortRange() {  // calculateShortRangeForces (p3mMethod.cpp:168-192)
    for (int i = 0; i < pm.N; ++i) {
      sr[i] = {};
      for (auto& s : slot[i]) s = {};
    }
    if (fast && q.y_sorting) {
      cm.fillSorted(pm.x);
      nextCell = 0;
      std::vector<std::thread> ts;
      for (int t = 0; t < std::max(1, nthreads); ++t) ts.emplace_back(&P3M::fastJob, this);
      for (auto& t : ts) t.join();
      return;
    }
    auto t0 = std::chrono::steady_clock::now();
    if (fillStride > 1 && q.y_sorting) {
      // timing sample: the reference's insertion sort on every fillStride-th particle (its
      // cost is quadratic in the cell populations, so the time is scaled by fillStride^2); the
      // complete lists for the pair pass come from the equivalent stable sort, untimed
      std::vector<V3<T>> xs;
      for (int i = 0; i < pm.N; i += fillStride) xs.push_back(pm.x[i]);
      ChainMesh<T> sub(&q, T(pm.p.H), int(xs.size()));
      sub.fill(xs, true);
      fillSec += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() *
                 double(fillStride) * double(fillStride);
      cm.fillSorted(pm.x);
    } else {
      cm.fill(pm.x, q.y_sorting != 0);
      fillSec += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    auto t1 = std::chrono::steady_clock::now();
    int th = std::max(1, nthreads);
    std::vector<std::thread> ts;
    for (int t = 0; t < th; ++t) ts.emplace_back(&P3M::threadJob, this, t, th);
    for (auto& t : ts) t.join();
    pairSec += std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
  }
  double fillSec = 0, pairSec = 0;
  int fillStride = 1;  // timing samples: see shortRange()
  void correct() {  // correctAccelerations (p3mMethod.cpp:50-57)
    for (int i = 0; i < pm.N; ++i) {
      V3<T> tot{};
      for (auto& s : slot[i]) tot += s;
      tot += sr[i];
      pm.a[i] += tot / pm.m[i];
    }
  }
};

template <typename T>
void exportState(PM<T>& pm, bool codeUnits, double* out) {
  int n = pm.N;
  for (int i = 0; i < n; ++i) {
    V3<T> x = pm.x[i], v = pm.v[i];
    if (codeUnits) {
      x = pm.H * x;
      v = (pm.H * v) / pm.DT;
    }
    out[3 * i] = x.x;
    out[3 * i + 1] = x.y;
    out[3 * i + 2] = x.z;
    out[3 * (n + i)] = v.x;
    out[3 * (n + i) + 1] = v.y;
    out[3 * (n + i) + 2] = v.z;
  }
}

/* ------------------------------------------------------------ diagnostics ---- */
// The quantities SimInfo computes (source/simInfo.cpp:50-127) at the point of the run loop
// where PMMethod::run / P3MMethod::run record them with collectDiagnostics
// (source/pmMethod.cpp:66-106, source/p3mMethod.cpp:69-130), every sum in double.  One record
// is 12 doubles, the layout of the C ABI's PMGB_DIAG_* indices:
//   0 potential energy  0.5 H^3 sum(rho_orig phi_orig) + sum(m Phi_ext(x))
//   1 kinetic energy    sum(0.5 m |v|^2), v = the half-step velocity
//   2-4 momentum        sum(m u), u = integer-step velocity v + a/2
//   5-7 angular mom.    sum(m x cross u)
//   8-10 expected mom.  initial momentum + DT sum over records of sum(m g_ext(x))
//   11 external part    sum(m Phi_ext(x))
struct DiagOut {
  double* out = nullptr;
  int cap = 0;
  int count = 0;
  double pexp[3] = {0, 0, 0};
};

// sphRadDecrField / sphRadDecrFieldPotential (source/externalFields.cpp:4-28) in double.
void extFieldPot(const orc_pm_params& p, double x, double y, double z, double g[3], double* phi) {
  g[0] = g[1] = g[2] = 0;
  *phi = 0;
  if (p.ext_kind != 1) return;
  const double dx = x - p.ext_cx, dy = y - p.ext_cy, dz = z - p.ext_cz;
  const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
  const double R = p.ext_R, M = p.ext_M, G = p.ext_G;
  const double gm = r > R ? -G * M / (r * r) : -(G * M / (R * R * R)) * r * (4 - 3 * r / R);
  if (r > 0) {
    g[0] = gm * dx / r;
    g[1] = gm * dy / r;
    g[2] = gm * dz / r;
  }
  const double u = r / R;
  *phi = r > R ? -G * M / r : G * M / R * (-2 + u * u * (2 - u));
}

// One record; pm.x, pm.v, pm.m and isv are in original units at this point of the loop.
template <typename T>
void diagRecord(const PM<T>& pm, const std::vector<V3<T>>& isv, DiagOut& d) {
  double ke = 0, P[3] = {0, 0, 0}, Lm[3] = {0, 0, 0}, F[3] = {0, 0, 0}, U = 0;
  for (int i = 0; i < pm.N; ++i) {
    const double m = pm.m[i];
    const double x = pm.x[i].x, y = pm.x[i].y, z = pm.x[i].z;
    const double vx = pm.v[i].x, vy = pm.v[i].y, vz = pm.v[i].z;
    const double ux = isv[i].x, uy = isv[i].y, uz = isv[i].z;
    ke += 0.5 * m * (vx * vx + vy * vy + vz * vz);
    P[0] += m * ux;
    P[1] += m * uy;
    P[2] += m * uz;
    Lm[0] += m * (y * uz - z * uy);
    Lm[1] += m * (z * ux - x * uz);
    Lm[2] += m * (x * uy - y * ux);
    double g[3], phi;
    extFieldPot(pm.p, x, y, z, g, &phi);
    F[0] += m * g[0];
    F[1] += m * g[1];
    F[2] += m * g[2];
    U += m * phi;
  }
  double mesh = 0;
  for (size_t id = 0; id < pm.L; ++id) mesh += double(pm.rhoReal[id]) * double(pm.pot[id].real());
  const double H = pm.p.H, DT = pm.p.DT, G = pm.p.G;
  const double kr = 1.0 / (DT * DT * 4 * std::numbers::pi * G), kp = H * H / (DT * DT);
  const double pe = 0.5 * (H * H * H) * mesh * kr * kp + U;
  for (int c = 0; c < 3; ++c) d.pexp[c] += DT * F[c];
  if (d.count < d.cap) {
    double* r = d.out + 12 * size_t(d.count);
    r[0] = pe;
    r[1] = ke;
    for (int c = 0; c < 3; ++c) {
      r[2 + c] = P[c];
      r[5 + c] = Lm[c];
      r[8 + c] = d.pexp[c];
    }
    r[11] = U;
  }
  ++d.count;
}

// PMMethod::run / P3MMethod::run without recording, with the diagnostics when diag != null
// (pmMethod.cpp:62-135, p3mMethod.cpp:59-166).
template <typename T>
void runLoop(PM<T>& pm, P3M<T>* p3m, int simLength, double* out, int* escaped,
             DiagOut* diag = nullptr) {
  auto force = [&]() {
    pm.step();
    if (p3m) {
      p3m->shortRange();
      p3m->correct();
    }
  };
  std::vector<V3<T>> isv;
  if (diag) {  // setInitialMomentum: integerStepVelocity == velocity at construction
    isv.resize(pm.N);
    for (int i = 0; i < pm.N; ++i)
      for (int c = 0; c < 3; ++c)
        diag->pexp[c] += double(pm.m[i]) * double(c == 0 ? pm.v[i].x : c == 1 ? pm.v[i].y : pm.v[i].z);
  }
  const T H = pm.H, DT = pm.DT, G = pm.G;
  pm.toCode();
  pm.initGreen();
  force();
  for (int i = 0; i < pm.N; ++i) pm.v[i] += T(0.5) * pm.a[i];  // setHalfStepVelocities
  *escaped = 0;
  for (int t = 0; t <= simLength; ++t) {
    for (int i = 0; i < pm.N; ++i) pm.x[i] += pm.v[i];  // updatePositions
    if (diag)  // setIntegerStepVelocities, integerStepVelocitiesToOriginalUnits
      for (int i = 0; i < pm.N; ++i) isv[i] = (H * (pm.v[i] + T(0.5) * pm.a[i])) / DT;
    pm.statesToOriginal();
    if (diag) {
      for (int i = 0; i < pm.N; ++i) pm.m[i] = (H * H * H) / (DT * DT * 4 * PI<T> * G) * pm.m[i];
      diagRecord(pm, isv, *diag);
    }
    if (pm.escaped()) {
      *escaped = 1;
      exportState(pm, false, out);
      return;
    }
    pm.statesToCode();
    if (diag)
      for (int i = 0; i < pm.N; ++i) pm.m[i] = DT * DT * 4 * PI<T> * G / (H * H * H) * pm.m[i];
    force();
    for (int i = 0; i < pm.N; ++i) pm.v[i] += pm.a[i];  // updateVelocities
  }
  exportState(pm, true, out);
}

template <typename T>
int pmAccel(const orc_pm_params* p, int n, const float* state, const float* masses, double* acc,
            double* density, double* potential, double* green) {
  PM<T> pm(p, n, state, masses, 1);
  pm.toCode();
  pm.initGreen();
  pm.step();
  for (int i = 0; i < n; ++i) {
    acc[3 * i] = pm.a[i].x;
    acc[3 * i + 1] = pm.a[i].y;
    acc[3 * i + 2] = pm.a[i].z;
  }
  for (size_t id = 0; id < pm.L; ++id) {
    if (potential) potential[id] = pm.pot[id].real();
    if (green) green[id] = pm.green[id];
  }
  if (density) {  // the forward FFT overwrote the mesh in place: deposit again
    pm.spreadMass();
    for (size_t id = 0; id < pm.L; ++id) density[id] = pm.dens[id].real();
  }
  return 0;
}

template <typename T>
int p3mAccel(const orc_pm_params* p, const orc_p3m_params* q, int n, const float* state,
             const float* masses, double* acc, double* acc_sr, int nthreads) {
  PM<T> pm(p, n, state, masses, nthreads);
  P3M<T> p3m(q, pm, nthreads);
  p3m.fast = true;
  pm.toCode();
  pm.initGreen();
  pm.step();
  std::vector<V3<T>> apm = pm.a;
  p3m.shortRange();
  p3m.correct();
  for (int i = 0; i < n; ++i) {
    acc[3 * i] = pm.a[i].x;
    acc[3 * i + 1] = pm.a[i].y;
    acc[3 * i + 2] = pm.a[i].z;
    if (acc_sr) {
      acc_sr[3 * i] = double(pm.a[i].x) - double(apm[i].x);
      acc_sr[3 * i + 1] = double(pm.a[i].y) - double(apm[i].y);
      acc_sr[3 * i + 2] = double(pm.a[i].z) - double(apm[i].z);
    }
  }
  return 0;
}

}  // namespace

extern "C" {

int port_pm_accel(int prec, const orc_pm_params* p, int n, const float* state,
                  const float* masses, double* acc, double* density, double* potential,
                  double* green) {
  return prec ? pmAccel<double>(p, n, state, masses, acc, density, potential, green)
              : pmAccel<float>(p, n, state, masses, acc, density, potential, green);
}

int port_p3m_accel(int prec, const orc_pm_params* p, const orc_p3m_params* q, int n,
                   const float* state, const float* masses, double* acc, double* acc_sr,
                   int nthreads) {
  return prec ? p3mAccel<double>(p, q, n, state, masses, acc, acc_sr, nthreads)
              : p3mAccel<float>(p, q, n, state, masses, acc, acc_sr, nthreads);
}

int port_pm_run(int prec, const orc_pm_params* p, int n, const float* state,
                const float* masses, int sim_length, double* state_out, int* escaped,
                double* diag, int diag_cap, int* diag_count) {
  DiagOut d;
  d.out = diag;
  d.cap = diag ? diag_cap : 0;
  DiagOut* dp = diag ? &d : nullptr;
  if (prec) {
    PM<double> pm(p, n, state, masses, 1);
    runLoop<double>(pm, nullptr, sim_length, state_out, escaped, dp);
  } else {
    PM<float> pm(p, n, state, masses, 1);
    runLoop<float>(pm, nullptr, sim_length, state_out, escaped, dp);
  }
  if (diag_count) *diag_count = d.count;
  return 0;
}

int port_p3m_run(int prec, const orc_pm_params* p, const orc_p3m_params* q, int n,
                 const float* state, const float* masses, int sim_length, double* state_out,
                 int* escaped, int nthreads, double* diag, int diag_cap, int* diag_count) {
  DiagOut d;
  d.out = diag;
  d.cap = diag ? diag_cap : 0;
  DiagOut* dp = diag ? &d : nullptr;
  if (prec) {
    PM<double> pm(p, n, state, masses, nthreads);
    P3M<double> p3m(q, pm, nthreads);
    p3m.fast = true;
    runLoop<double>(pm, &p3m, sim_length, state_out, escaped, dp);
  } else {
    PM<float> pm(p, n, state, masses, nthreads);
    P3M<float> p3m(q, pm, nthreads);
    p3m.fast = true;
    runLoop<float>(pm, &p3m, sim_length, state_out, escaped, dp);
  }
  if (diag_count) *diag_count = d.count;
  return 0;
}

int port_chaining_mesh(const orc_p3m_params* q, float H, int n, const float* pos_code,
                       int y_sorting, int* order, int* counts, int* dims) {
  ChainMesh<float> cm(q, H, n);
  dims[0] = cm.Mx;
  dims[1] = cm.My;
  dims[2] = cm.Mz;
  if (!order) return 0;
  std::vector<V3<float>> x(n);
  for (int i = 0; i < n; ++i) x[i] = {pos_code[3 * i], pos_code[3 * i + 1], pos_code[3 * i + 2]};
  cm.fill(x, y_sorting != 0);
  int k = 0;
  for (int c = 0; c < cm.size; ++c) {
    int cnt = 0;
    for (int i = cm.hoc[c]; i >= 0; i = cm.next[i]) {
      order[k++] = i;
      ++cnt;
    }
    counts[c] = cnt;
  }
  return 0;
}

int port_pp_accel(int n, const double* pos, const double* masses, double G, double eps, int m,
                  const int* idx, double periodic_L, double* acc, int nthreads) {
  parallel_for(m, nthreads, [&](int b, int e) {
    for (int k = b; k < e; ++k) {
      int i = idx[k];
      double ax = 0, ay = 0, az = 0;
      for (int j = 0; j < n; ++j) {
        if (j == i) continue;
        double dx = pos[3 * i] - pos[3 * j], dy = pos[3 * i + 1] - pos[3 * j + 1],
               dz = pos[3 * i + 2] - pos[3 * j + 2];
        if (periodic_L > 0) {
          dx -= periodic_L * std::nearbyint(dx / periodic_L);
          dy -= periodic_L * std::nearbyint(dy / periodic_L);
          dz -= periodic_L * std::nearbyint(dz / periodic_L);
        }
        double r2 = dx * dx + dy * dy + dz * dz + eps * eps;
        double s = -G * masses[j] / (r2 * std::sqrt(r2));
        ax += s * dx;
        ay += s * dy;
        az += s * dz;
      }
      acc[3 * k] = ax;
      acc[3 * k + 1] = ay;
      acc[3 * k + 2] = az;
    }
  });
  return 0;
}

int port_p3m_accel_targets(int prec, const orc_pm_params* p, const orc_p3m_params* q, int n,
                           const float* state, const float* masses, int m, const int* idx,
                           double* acc, int nthreads) {
  auto body = [&](auto tag) {
    using T = decltype(tag);
    PM<T> pm(p, n, state, masses, nthreads);
    P3M<T> p3m(q, pm, 1);
    pm.toCode();
    pm.initGreen();
    pm.step();
    // every pair within the cutoff lies in the same or adjacent chaining cells (cell side >=
    // cutoff), so a brute-force sum over the particles inside the chaining mesh is the
    // reference's pair set
    std::vector<char> inside(n);
    for (int j = 0; j < n; ++j) inside[j] = p3m.cm.cellOf(pm.x[j]) >= 0;
    parallel_for(m, nthreads, [&](int b, int e) {
      for (int k = b; k < e; ++k) {
        const int i = idx[k];
        V3<T> a = pm.a[i];
        if (inside[i]) {
          V3<T> s{};
          for (int j = 0; j < n; ++j) {
            if (j == i || !inside[j]) continue;
            V3<T> rij = pm.x[i] - pm.x[j];
            if (mag2(rij) >= p3m.re * p3m.re) continue;
            s += p3m.srForce(rij, pm.m[i], pm.m[j]);
          }
          a += s / pm.m[i];
        }
        acc[3 * k] = a.x;
        acc[3 * k + 1] = a.y;
        acc[3 * k + 2] = a.z;
      }
    });
  };
  if (prec) body(double{});
  else body(float{});
  return 0;
}

int port_sr_table(const orc_p3m_params* q, float H, float* table, float* delta_sq) {
  orc_pm_params p{};
  p.nx = p.ny = p.nz = 1;
  p.H = H;
  p.DT = 1;
  p.G = 1;
  float st[6] = {0, 0, 0, 0, 0, 0}, ms[1] = {1};
  PM<float> pm(&p, 1, st, ms, 1);
  orc_p3m_params qq = *q;
  qq.use_table = 1;
  P3M<float> p3m(&qq, pm, 1);
  for (int i = 0; i < 500; ++i) table[i] = p3m.table[i];
  *delta_sq = p3m.delta2;
  return 0;
}

int port_time_steps(const orc_pm_params* p, const orc_p3m_params* q, int n, const float* state,
                    const float* masses, int steps, int nthreads, int pair_stride, double* out4) {
  return port_time_steps2(p, q, n, state, masses, steps, nthreads, pair_stride, 1, out4, nullptr);
}

int port_time_steps2(const orc_pm_params* p, const orc_p3m_params* q, int n, const float* state,
                     const float* masses, int steps, int nthreads, int pair_stride,
                     int fill_stride, double* out4, double* wall) {
  // Times `steps` iterations of the run loop body (drift, force, kick) in float with nthreads
  // host threads.  With pair_stride S > 1 only every S-th particle of each cell list is an
  // i-particle of the pair pass (its j loops are complete), and the pair time is scaled by S.
  // out4 = {estimated seconds per full step, PM seconds, cell-list seconds, pair seconds as
  // measured (sampled)}, all per step.
  PM<float> pm(p, n, state, masses, nthreads);
  std::unique_ptr<P3M<float>> p3m;
  if (q) {
    p3m = std::make_unique<P3M<float>>(q, pm, nthreads);
    p3m->pairStride = std::max(1, pair_stride);
    p3m->fillStride = std::max(1, fill_stride);
  }
  pm.toCode();
  pm.initGreen();
  double pmSec = 0;
  const auto w0 = std::chrono::steady_clock::now();
  for (int t = 0; t < steps; ++t) {
    for (int i = 0; i < n; ++i) pm.x[i] += pm.v[i];
    pm.statesToOriginal();
    pm.statesToCode();
    auto t0 = std::chrono::steady_clock::now();
    pm.step();
    pmSec += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (p3m) {
      p3m->shortRange();
      p3m->correct();
    }
    for (int i = 0; i < n; ++i) pm.v[i] += pm.a[i];
  }
  if (wall) *wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - w0).count();
  const int k = std::max(1, steps);
  const double fill = p3m ? p3m->fillSec / k : 0.0, pair = p3m ? p3m->pairSec / k : 0.0;
  out4[1] = pmSec / k;
  out4[2] = fill;
  out4[3] = pair;
  out4[0] = out4[1] + fill + pair * (p3m ? p3m->pairStride : 1);
  return 0;
}

}  // extern "C"
