// Host-side set-up of the element update: synthetic periodic cube mesh, face relations,
// materials, star matrices and flux solvers (float64 arithmetic, stored as float32).
//
// Conventions followed:
//   FACE2NODES, normals, tangents   src/Geometry/MeshTools.cpp:21-69
//   neighbour side / orientation    src/Geometry/PUMLReader.cpp:151-163, 405-427
//   Jacobian of the reference map   src/Numerical/Transformation.cpp:66-108
//   A^T, B^T, C^T, Godunov state    src/Equations/elastic/Model/ElasticSetup.h:27-180
//   face rotation T, Tinv           src/Numerical/Transformation.cpp:110-290
//   star matrices, flux solvers     src/Initializer/Model/CellLocalMatrices.cpp:46-296
//                                   codegen/kernels/aderdg.py:226-246
//   CFL time step                   src/Initializer/TimeStepping/GlobalTimestep.cpp:27-47
#include "internal.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <string>
#include <stdexcept>
#include <vector>

namespace sei {

namespace {

const int kFace2Nodes[4][3] = {{0, 2, 1}, {0, 1, 3}, {0, 3, 2}, {1, 2, 3}};

// 5-tetrahedron split of a unit cube (even parity); odd cubes use the mirror image in x.
const int kEvenTets[5][4][3] = {
    {{0, 0, 0}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}},
    {{1, 0, 0}, {0, 0, 0}, {1, 1, 0}, {1, 0, 1}},
    {{0, 1, 0}, {0, 0, 0}, {1, 1, 0}, {0, 1, 1}},
    {{0, 0, 1}, {0, 0, 0}, {1, 0, 1}, {0, 1, 1}},
    {{1, 1, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}},
};

using Vec3 = std::array<double, 3>;
using Mat9 = std::array<double, 81>;  // row-major [i][j] = view (i, j)

Vec3 sub(const Vec3& a, const Vec3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
Vec3 cross(const Vec3& a, const Vec3& b) {
  return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
double dot(const Vec3& a, const Vec3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
double norm(const Vec3& a) { return std::sqrt(dot(a, a)); }
Vec3 scale(const Vec3& a, double s) { return {a[0] * s, a[1] * s, a[2] * s}; }

// splitmix64: portable, seeded uniform numbers.
struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform(double lo, double hi) { return lo + (hi - lo) * ((next() >> 11) * (1.0 / 9007199254740992.0)); }
};

void coefficientMatrixT(double rho, double mu, double lam, int dim, Mat9& m) {
  m.fill(0.0);
  const double l2m = lam + 2.0 * mu, ri = 1.0 / rho;
  auto at = [&](int i, int j) -> double& { return m[i * 9 + j]; };
  if (dim == 0) {
    at(6, 0) = -l2m; at(6, 1) = -lam; at(6, 2) = -lam; at(7, 3) = -mu; at(8, 5) = -mu;
    at(0, 6) = -ri; at(3, 7) = -ri; at(5, 8) = -ri;
  } else if (dim == 1) {
    at(7, 0) = -lam; at(7, 1) = -l2m; at(7, 2) = -lam; at(6, 3) = -mu; at(8, 4) = -mu;
    at(1, 7) = -ri; at(3, 6) = -ri; at(4, 8) = -ri;
  } else {
    at(8, 0) = -lam; at(8, 1) = -lam; at(8, 2) = -l2m; at(7, 4) = -mu; at(6, 5) = -mu;
    at(2, 8) = -ri; at(5, 6) = -ri; at(4, 7) = -ri;
  }
}

// Solves A X = Bm (9x9, row-major) by LU with partial pivoting; Bm is overwritten with X.
void solve9(Mat9 a, Mat9& bm) {
  int piv[9];
  for (int i = 0; i < 9; ++i) piv[i] = i;
  for (int c = 0; c < 9; ++c) {
    int p = c;
    for (int r = c + 1; r < 9; ++r)
      if (std::fabs(a[r * 9 + c]) > std::fabs(a[p * 9 + c])) p = r;
    if (a[p * 9 + c] == 0.0) throw std::runtime_error("singular eigenvector basis in Godunov state");
    if (p != c) {
      for (int j = 0; j < 9; ++j) {
        std::swap(a[c * 9 + j], a[p * 9 + j]);
        std::swap(bm[c * 9 + j], bm[p * 9 + j]);
      }
    }
    for (int r = c + 1; r < 9; ++r) {
      const double f = a[r * 9 + c] / a[c * 9 + c];
      if (f == 0.0) continue;
      for (int j = c; j < 9; ++j) a[r * 9 + j] -= f * a[c * 9 + j];
      for (int j = 0; j < 9; ++j) bm[r * 9 + j] -= f * bm[c * 9 + j];
    }
  }
  for (int c = 8; c >= 0; --c) {
    for (int j = 0; j < 9; ++j) {
      double s = bm[c * 9 + j];
      for (int k = c + 1; k < 9; ++k) s -= a[c * 9 + k] * bm[k * 9 + j];
      bm[c * 9 + j] = s / a[c * 9 + c];
    }
  }
}

// Transposed Godunov states of a regular face; materials (rho, mu, lambda).
void godunovState(const double* loc, const double* nb, Mat9& local, Mat9& neigh) {
  const double rl = loc[0], ml = loc[1], ll = loc[2];
  const double rn = nb[0], mn = nb[1], ln = nb[2];
  Mat9 r{};
  auto R = [&](int i, int j) -> double& { return r[i * 9 + j]; };
  R(0, 0) = ll + 2 * ml; R(1, 0) = ll; R(2, 0) = ll; R(6, 0) = std::sqrt((ll + 2 * ml) / rl);
  R(3, 1) = ml; R(7, 1) = std::sqrt(ml / rl);
  R(5, 2) = ml; R(8, 2) = std::sqrt(ml / rl);
  R(4, 3) = ll + 2 * ml; R(1, 4) = ll + 2 * ml; R(2, 5) = ll + 2 * ml;
  R(5, 6) = mn; R(8, 6) = -std::sqrt(mn / rn);
  R(3, 7) = mn; R(7, 7) = -std::sqrt(mn / rn);
  R(0, 8) = ln + 2 * mn; R(1, 8) = ln; R(2, 8) = ln; R(6, 8) = -std::sqrt((ln + 2 * mn) / rn);
  Mat9 rt{}, rhs{};
  for (int i = 0; i < 9; ++i)
    for (int j = 0; j < 9; ++j) rt[i * 9 + j] = r[j * 9 + i];
  // rhs = chi R^T with chi = diag(1, 1, 1, 0, ...): the first three rows of R^T.
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 9; ++j) rhs[i * 9 + j] = rt[i * 9 + j];
  solve9(rt, rhs);
  for (int i = 0; i < 9; ++i)
    for (int j = 0; j < 9; ++j) {
      neigh[i * 9 + j] = rhs[i * 9 + j];
      local[i * 9 + j] = (i == j ? 1.0 : 0.0) - rhs[i * 9 + j];
    }
}

// Transposed Godunov state of a free-surface face (src/Model/Common.h:319-364, elastic case):
// S = -(R21 R11^-1) from the traction rows (0, 3, 5) and velocity rows (6, 7, 8) of the first three
// eigenvectors, set as local(t_i, v_j) = S(j, i), and the identity on the velocities.  R11 and R21
// are diagonal for an isotropic solid.  The neighbour state is unused (no neighbour flux); it is zero.
void freeSurfaceState(const double* loc, Mat9& local, Mat9& neigh) {
  const double r = loc[0], mu = loc[1], lam = loc[2];
  local.fill(0.0);
  neigh.fill(0.0);
  local[0 * 9 + 6] = -(std::sqrt((lam + 2 * mu) / r) * (1.0 / (lam + 2 * mu)));
  local[3 * 9 + 7] = -(std::sqrt(mu / r) * (1.0 / mu));
  local[5 * 9 + 8] = -(std::sqrt(mu / r) * (1.0 / mu));
  local[6 * 9 + 6] = local[7 * 9 + 7] = local[8 * 9 + 8] = 1.0;
}

// Godunov states of face f of cell c: the free-surface state on a free-surface boundary, else the
// regular state with the neighbour's material (the cell's own on a boundary face,
// CellLocalMatrices.cpp:170-177).
void faceGodunov(const HostMesh& m, int64_t c, int f, Mat9& local, Mat9& neigh) {
  const double* mat = &m.material[c * 3];
  if (!m.bc.empty() && m.bc[c * 4 + f] == 1) {
    freeSurfaceState(mat, local, neigh);
    return;
  }
  const int32_t nb = m.nbr[c * 4 + f];
  godunovState(mat, nb >= 0 ? &m.material[(int64_t)nb * 3] : mat, local, neigh);
}

void rotation(const Vec3& n, const Vec3& s, const Vec3& t, Mat9& T, Mat9& Ti) {
  T.fill(0.0);
  Ti.fill(0.0);
  auto at = [](Mat9& m, int i, int j) -> double& { return m[i * 9 + j]; };
  const double nx = n[0], ny = n[1], nz = n[2], sx = s[0], sy = s[1], sz = s[2], tx = t[0], ty = t[1], tz = t[2];
  const double tcol[6][6] = {
      {nx * nx, ny * ny, nz * nz, ny * nx, nz * ny, nz * nx},
      {sx * sx, sy * sy, sz * sz, sy * sx, sz * sy, sz * sx},
      {tx * tx, ty * ty, tz * tz, ty * tx, tz * ty, tz * tx},
      {2 * nx * sx, 2 * ny * sy, 2 * nz * sz, ny * sx + nx * sy, nz * sy + ny * sz, nz * sx + nx * sz},
      {2 * sx * tx, 2 * sy * ty, 2 * sz * tz, sy * tx + sx * ty, sz * ty + sy * tz, sz * tx + sx * tz},
      {2 * nx * tx, 2 * ny * ty, 2 * nz * tz, ny * tx + nx * ty, nz * ty + ny * tz, nz * tx + nx * tz}};
  const double icol[6][6] = {
      {nx * nx, sx * sx, tx * tx, nx * sx, sx * tx, nx * tx},
      {ny * ny, sy * sy, ty * ty, ny * sy, sy * ty, ny * ty},
      {nz * nz, sz * sz, tz * tz, nz * sz, sz * tz, nz * tz},
      {2 * ny * nx, 2 * sy * sx, 2 * ty * tx, ny * sx + nx * sy, sy * tx + sx * ty, ny * tx + nx * ty},
      {2 * nz * ny, 2 * sz * sy, 2 * tz * ty, nz * sy + ny * sz, sz * ty + sy * tz, nz * ty + ny * tz},
      {2 * nz * nx, 2 * sz * sx, 2 * tz * tx, nz * sx + nx * sz, sz * tx + sx * tz, nz * tx + nx * tz}};
  for (int c = 0; c < 6; ++c)
    for (int r = 0; r < 6; ++r) {
      at(T, r, c) = tcol[c][r];
      at(Ti, r, c) = icol[c][r];
    }
  for (int i = 0; i < 3; ++i) {
    at(T, 6 + i, 6) = n[i];
    at(T, 6 + i, 7) = s[i];
    at(T, 6 + i, 8) = t[i];
    at(Ti, 6, 6 + i) = n[i];
    at(Ti, 7, 6 + i) = s[i];
    at(Ti, 8, 6 + i) = t[i];
  }
}

// out(i, j) = s * sum_{k, l} Tinv(k, i) (Qgod A~^T)(k, l) T(j, l), written column-major (i + 9 j) as float.
void fluxSolver(double s, const Mat9& Ti, const Mat9& qgod, const Mat9& at, const Mat9& T, float* out) {
  Mat9 qa{}, tmp{};
  for (int k = 0; k < 9; ++k)
    for (int l = 0; l < 9; ++l) {
      double v = 0;
      for (int q = 0; q < 9; ++q) v += qgod[k * 9 + q] * at[q * 9 + l];
      qa[k * 9 + l] = v;
    }
  for (int i = 0; i < 9; ++i)
    for (int l = 0; l < 9; ++l) {
      double v = 0;
      for (int k = 0; k < 9; ++k) v += Ti[k * 9 + i] * qa[k * 9 + l];
      tmp[i * 9 + l] = v;
    }
  for (int i = 0; i < 9; ++i)
    for (int j = 0; j < 9; ++j) {
      double v = 0;
      for (int l = 0; l < 9; ++l) v += tmp[i * 9 + l] * T[j * 9 + l];
      out[i + 9 * j] = static_cast<float>(s * v);
    }
}

}  // namespace

// The local-time-stepping profile: shares of the banded direction's intervals in the four bands,
// the edge of each band and the edge of the other two directions (units of h).  A cube w x L x L (w << L) splits into tets of
// inradius about (w / 2) / (1 + w / L), so the band edges are set for inradii 1.3 2^b times that
// of band 0: with the material's +-10 % wave speeds every tet of band b then has a CFL step in
// [2^b, 2^(b+1)) times the smallest one, i.e. lies in rate-2 cluster b.
constexpr double kLtsBandShare[4] = {0.60, 0.25, 0.10, 0.05};
constexpr double kLtsBandEdge[4] = {1.0, 2.736, 5.98, 14.7};
constexpr double kLtsCrossEdge = 32.0;

void buildPeriodicCube(const sei_cube_params& p, HostMesh& m) {
  // Even counts keep the alternating 5-tet split conforming across cubes; at least 4 cubes per
  // direction keep the periodically identified faces distinct.
  if (p.nx < 4 || p.ny < 4 || p.nz < 4 || p.nx % 2 || p.ny % 2 || p.nz % 2)
    throw std::invalid_argument("periodic cube needs even cube counts >= 4 in every direction");
  if (!(p.h > 0) || !(p.rho > 0) || !(p.vp > 0) || !(p.vs > 0) || p.perturb < 0 || p.perturb >= 0.5)
    throw std::invalid_argument("invalid cube geometry or material");
  const int64_t ncubes = (int64_t)p.nx * p.ny * p.nz;
  // vertex positions along each direction: cumulative cube edges (uniform h, or log-uniform in
  // [h, grading h] from the seed); index nx (ny, nz) is the periodic image of 0
  std::vector<double> pos[3];
  {
    Rng grng(p.seed ^ 0x9E3779B97F4A7C15ull);
    const int cnt[3] = {p.nx, p.ny, p.nz};
    for (int d = 0; d < 3; ++d) {
      pos[d].assign(cnt[d] + 1, 0.0);
      if (p.lts_profile == 1 && p.grading >= 8.0) {
        // the direction with the most intervals (x on ties): bands b = 0..3 of the edge on fixed
        // shares of the intervals, rising then falling once (band sequence 0 .. 3 .. 0, each band
        // split between the two slopes), so neighbouring cubes lie in the same or adjacent bands
        // also across the periodic boundary; the other two directions: one long edge, so the
        // banded edge bounds each tet's time step and rate-2 clustering follows the bands
        const int banded = cnt[2] > cnt[1] && cnt[2] > cnt[0] ? 2 : (cnt[1] > cnt[0] ? 1 : 0);
        if (d != banded) {
          for (int i = 0; i < cnt[d]; ++i) pos[d][i + 1] = pos[d][i] + p.h * kLtsCrossEdge;
          continue;
        }
        int count[4], used = 0;
        for (int b = 3; b >= 1; --b) {
          count[b] = std::max(1, (int)std::lround(kLtsBandShare[b] * cnt[d]));
          used += count[b];
        }
        count[0] = std::max(1, cnt[d] - used);
        std::vector<int> band;
        for (int b = 0; b < 4; ++b)
          for (int k = 0; k < (count[b] + 1) / 2; ++k) band.push_back(b);
        for (int b = 3; b >= 0; --b)
          for (int k = 0; k < count[b] / 2; ++k) band.push_back(b);
        band.resize(cnt[d], 0);
        for (int i = 0; i < cnt[d]; ++i) pos[d][i + 1] = pos[d][i] + p.h * kLtsBandEdge[band[i]];
        continue;
      }
      for (int i = 0; i < cnt[d]; ++i) {
        const double w = p.grading > 1.0 ? p.h * std::exp(grng.uniform(0.0, std::log(p.grading))) : p.h;
        pos[d][i + 1] = pos[d][i] + w;
      }
    }
  }
  m.fault_x = (p.fault_plane >= 0 && p.fault_plane <= p.nx) ? pos[0][p.fault_plane] : 0.0;
  m.n = ncubes * 5;
  m.topo.resize(m.n * 4);
  m.coords.resize(m.n * 12);
  m.material.resize(m.n * 3);
  int tets[2][5][4][3];
  for (int par = 0; par < 2; ++par)
    for (int t = 0; t < 5; ++t) {
      for (int v = 0; v < 4; ++v) {
        tets[par][t][v][0] = par ? 1 - kEvenTets[t][v][0] : kEvenTets[t][v][0];
        tets[par][t][v][1] = kEvenTets[t][v][1];
        tets[par][t][v][2] = kEvenTets[t][v][2];
      }
      Vec3 a{}, b{}, c{}, d{};
      for (int k = 0; k < 3; ++k) {
        a[k] = tets[par][t][0][k];
        b[k] = tets[par][t][1][k];
        c[k] = tets[par][t][2][k];
        d[k] = tets[par][t][3][k];
      }
      if (dot(cross(sub(b, a), sub(c, a)), sub(d, a)) < 0)
        for (int k = 0; k < 3; ++k) std::swap(tets[par][t][2][k], tets[par][t][3][k]);
    }
  // Cell order: the cubes of each parity are listed pencil by pencil (pencils of 8 x 8 cubes in
  // x, y, all of z; pencils in serpentine order over the x-y plane; (k, j, i) order inside a
  // pencil) and cut into chunks of 32; chunk c emits, for parity 0 then 1 and tet type 0..4, the
  // 32 cells of that type.  A 32-cell CTA therefore holds one tet type (uniform face relations).
  // Every cube's neighbours lie within one pencil (<= 64 cubes away in z) or in the adjacent
  // pencil, so the four reads of each time-integrated block by the neighbour kernel fall within
  // a few thousand cubes of each other and are served from L2.
  constexpr int kPencil = 8;
  std::vector<std::array<int, 3>> cubes[2];
  const int npx = (p.nx + kPencil - 1) / kPencil, npy = (p.ny + kPencil - 1) / kPencil;
  for (int pj = 0; pj < npy; ++pj)
    for (int pq = 0; pq < npx; ++pq) {
      const int pi = (pj % 2) ? npx - 1 - pq : pq;
      for (int k = 0; k < p.nz; ++k)
        for (int j = pj * kPencil; j < std::min(p.ny, (pj + 1) * kPencil); ++j)
          for (int i = pi * kPencil; i < std::min(p.nx, (pi + 1) * kPencil); ++i)
            cubes[(i + j + k) % 2].push_back({i, j, k});
    }
  const size_t chunks = (cubes[0].size() + 31) / 32;
  int64_t cell = 0;
  for (size_t ch = 0; ch < chunks; ++ch)
    for (int par = 0; par < 2; ++par)
      for (int t = 0; t < 5; ++t)
        for (size_t mi = ch * 32; mi < std::min(cubes[par].size(), ch * 32 + 32); ++mi) {
          const int i = cubes[par][mi][0], j = cubes[par][mi][1], k = cubes[par][mi][2];
          {
            for (int v = 0; v < 4; ++v) {
              const int gi = i + tets[par][t][v][0], gj = j + tets[par][t][v][1], gk = k + tets[par][t][v][2];
              m.topo[cell * 4 + v] = (gi % p.nx) + (int64_t)p.nx * ((gj % p.ny) + (int64_t)p.ny * (gk % p.nz));
              m.coords[cell * 12 + v * 3 + 0] = pos[0][gi];
              m.coords[cell * 12 + v * 3 + 1] = pos[1][gj];
              m.coords[cell * 12 + v * 3 + 2] = pos[2][gk];
            }
            ++cell;
          }
        }
  Rng rng(p.seed);
  for (int64_t c = 0; c < m.n; ++c) {
    double rho = p.rho, vp = p.vp, vs = p.vs;
    if (p.perturb > 0) {
      rho *= rng.uniform(1 - p.perturb, 1 + p.perturb);
      vp *= rng.uniform(1 - p.perturb, 1 + p.perturb);
      vs *= rng.uniform(1 - p.perturb, 1 + p.perturb);
    }
    const double mu = rho * vs * vs, lam = rho * vp * vp - 2 * mu;
    if (!(lam > -2.0 / 3.0 * mu)) throw std::invalid_argument("material perturbation gives a non-physical cell");
    m.material[c * 3 + 0] = rho;
    m.material[c * 3 + 1] = mu;
    m.material[c * 3 + 2] = lam;
  }
  computeFaceRelations(m);
}

void computeFaceRelations(HostMesh& m) {
  m.nbr.assign(m.n * 4, -1);
  m.side.assign(m.n * 4, 0);
  m.orient.assign(m.n * 4, 0);
  m.ftype.assign(m.n * 4, 2);
  std::map<std::array<int64_t, 3>, std::array<int64_t, 2>> faces;
  for (int64_t c = 0; c < m.n; ++c)
    for (int f = 0; f < 4; ++f) {
      std::array<int64_t, 3> key{m.topo[c * 4 + kFace2Nodes[f][0]], m.topo[c * 4 + kFace2Nodes[f][1]],
                                 m.topo[c * 4 + kFace2Nodes[f][2]]};
      std::sort(key.begin(), key.end());
      auto it = faces.find(key);
      if (it == faces.end()) {
        faces.emplace(key, std::array<int64_t, 2>{c * 4 + f, -1});
      } else {
        if (it->second[1] != -1) throw std::runtime_error("non-manifold face in mesh");
        it->second[1] = c * 4 + f;
      }
    }
  for (const auto& kv : faces) {
    const int64_t a = kv.second[0], b = kv.second[1];
    if (b < 0) continue;
    for (int dir = 0; dir < 2; ++dir) {
      const int64_t cf = dir ? b : a, df = dir ? a : b;
      const int64_t c = cf / 4, d = df / 4;
      const int f = (int)(cf % 4), j = (int)(df % 4);
      m.nbr[cf] = (int32_t)d;
      m.side[cf] = (int8_t)j;
      m.ftype[cf] = 0;
      const int64_t first = m.topo[c * 4 + kFace2Nodes[f][0]];
      int h = -1;
      for (int k = 0; k < 3; ++k)
        if (m.topo[d * 4 + kFace2Nodes[j][k]] == first) h = k;
      if (h < 0) throw std::runtime_error("face orientation not found");
      m.orient[cf] = (int8_t)h;
    }
  }
}

void buildOperators(const HostMesh& m, std::vector<float>& star, std::vector<float>& aplus,
                    std::vector<float>& aminus) {
  star.assign(m.n * 3 * 81, 0.f);
  aplus.assign(m.n * 4 * 81, 0.f);
  aminus.assign(m.n * 4 * 81, 0.f);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < m.n; ++c) {
    const double* mat = &m.material[c * 3];
    Mat9 at[3];
    for (int d = 0; d < 3; ++d) coefficientMatrixT(mat[0], mat[1], mat[2], d, at[d]);
    Vec3 v[4];
    for (int k = 0; k < 4; ++k) v[k] = {m.coords[c * 12 + k * 3], m.coords[c * 12 + k * 3 + 1], m.coords[c * 12 + k * 3 + 2]};
    // Rows of the inverse of J = [v1-v0, v2-v0, v3-v0] (columns) are grad xi, grad eta, grad zeta.
    const Vec3 e1 = sub(v[1], v[0]), e2 = sub(v[2], v[0]), e3 = sub(v[3], v[0]);
    const double det = dot(e1, cross(e2, e3));
    const Vec3 g[3] = {scale(cross(e2, e3), 1.0 / det), scale(cross(e3, e1), 1.0 / det),
                       scale(cross(e1, e2), 1.0 / det)};
    for (int e = 0; e < 3; ++e)
      for (int i = 0; i < 9; ++i)
        for (int j = 0; j < 9; ++j)
          star[(c * 3 + e) * 81 + i + 9 * j] =
              static_cast<float>(g[e][0] * at[0][i * 9 + j] + g[e][1] * at[1][i * 9 + j] + g[e][2] * at[2][i * 9 + j]);
    const double volume = std::fabs(det) / 6.0;
    for (int f = 0; f < 4; ++f) {
      const Vec3 a = v[kFace2Nodes[f][0]], b = v[kFace2Nodes[f][1]], cc = v[kFace2Nodes[f][2]];
      Vec3 nrm = cross(sub(b, a), sub(cc, a));
      const double area = 0.5 * norm(nrm);
      Vec3 t1 = sub(b, a);
      Vec3 t2 = cross(nrm, t1);
      nrm = scale(nrm, 1.0 / norm(nrm));
      t1 = scale(t1, 1.0 / norm(t1));
      t2 = scale(t2, 1.0 / norm(t2));
      Mat9 qgl, qgn, T, Ti;
      faceGodunov(m, c, f, qgl, qgn);
      rotation(nrm, t1, t2, T, Ti);
      const double fs = -2.0 * area / (6.0 * volume);
      const bool dr = m.ftype[c * 4 + f] == 1;
      fluxSolver(dr ? 0.0 : fs, Ti, qgl, at[0], T, &aplus[(c * 4 + f) * 81]);
      fluxSolver(fs, Ti, qgn, at[0], T, &aminus[(c * 4 + f) * 81]);
    }
  }
}

void fitAttenuation(double qp, double qs, double freqCentral, double freqRatio, double& mu, double& lam,
                    double omega[kMechanisms], double theta[kMechanisms][3]) {
  // Attenuation.h:24-104: kMax = 2 L - 1 frequencies log-spaced over the band; least-squares
  // weights alpha (P) and beta (S); unrelaxed moduli from the phase at the central frequency.
  constexpr int L = kMechanisms, K = 2 * kMechanisms - 1;
  const double pi = 3.14159265358979323846;
  const double w0 = 2 * pi * freqCentral, wmin = w0 / std::sqrt(freqRatio);
  double w[K];
  for (int i = 0; i < K; ++i) w[i] = std::exp(std::log(wmin) + (double)i / (K - 1) * std::log(freqRatio));
  for (int i = 0; i < L; ++i) omega[i] = w[2 * i];
  auto lsq = [&](double q, double* x) {
    // columns a_j(i) = (w_2j w_i + w_2j^2 / q) / (w_2j^2 + w_i^2); solve min |A x - 1/q| by Gram-Schmidt QR
    double a[L][K], r[L][L] = {}, b[K];
    for (int i = 0; i < K; ++i) b[i] = 1.0 / q;
    for (int j = 0; j < L; ++j)
      for (int i = 0; i < K; ++i) {
        const double wj = w[2 * j];
        a[j][i] = (wj * w[i] + wj * wj / q) / (wj * wj + w[i] * w[i]);
      }
    for (int j = 0; j < L; ++j) {
      for (int p = 0; p < j; ++p) {
        double d = 0;
        for (int i = 0; i < K; ++i) d += a[p][i] * a[j][i];
        r[p][j] = d;
        for (int i = 0; i < K; ++i) a[j][i] -= d * a[p][i];
      }
      double nrm = 0;
      for (int i = 0; i < K; ++i) nrm += a[j][i] * a[j][i];
      nrm = std::sqrt(nrm);
      r[j][j] = nrm;
      for (int i = 0; i < K; ++i) a[j][i] /= nrm;
    }
    double y[L];
    for (int j = 0; j < L; ++j) {
      double d = 0;
      for (int i = 0; i < K; ++i) d += a[j][i] * b[i];
      y[j] = d;
    }
    for (int j = L - 1; j >= 0; --j) {
      double s = y[j];
      for (int p = j + 1; p < L; ++p) s -= r[j][p] * x[p];
      x[j] = s / r[j][j];
    }
  };
  double alpha[L], beta[L];
  lsq(qp, alpha);
  lsq(qs, beta);
  double p1 = 1, p2 = 0, s1 = 1, s2 = 0;
  for (int i = 0; i < L; ++i) {
    const double r = w0 / w[2 * i], d = 1 + r * r;
    p1 -= alpha[i] / d;
    p2 += alpha[i] * r / d;
    s1 -= beta[i] / d;
    s2 += beta[i] * r / d;
  }
  const double rp = std::sqrt(p1 * p1 + p2 * p2), rs = std::sqrt(s1 * s1 + s2 * s2);
  const double varP = (lam + 2 * mu) * (rp + p1) / (2 * rp * rp);
  const double varMu = mu * (rs + s1) / (2 * rs * rs);
  for (int i = 0; i < L; ++i) {
    const double t1 = -varP * alpha[i], t2 = -2.0 * varMu * beta[i];
    theta[i][0] = t1;
    theta[i][1] = t1 - t2;
    theta[i][2] = t2;
  }
  mu = varMu;
  lam = varP - 2 * varMu;
}

void buildViscoOperators(const HostMesh& m, std::vector<float>& grad, std::vector<float>& wplus,
                         std::vector<float>& wminus) {
  // The memory variables of mechanism l couple to the velocities through -omega_l C_x
  // (ViscoelasticSetup.h:26-48 with omega = 1) and receive the flux omega_l W, with
  // W[i][j] = s sum_k Tinv(k, i) sum_l (Qgod C_0)(k, l) T6(j, l) (aderdg.py:226-246; T6 the
  // stress block of T, which also rotates every mechanism's memory variables).
  grad.assign(m.n * 9, 0.f);
  wplus.assign(m.n * 4 * 54, 0.f);
  wminus.assign(m.n * 4 * 54, 0.f);
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < m.n; ++c) {
    Vec3 v[4];
    for (int k = 0; k < 4; ++k) v[k] = {m.coords[c * 12 + k * 3], m.coords[c * 12 + k * 3 + 1], m.coords[c * 12 + k * 3 + 2]};
    const Vec3 e1 = sub(v[1], v[0]), e2 = sub(v[2], v[0]), e3 = sub(v[3], v[0]);
    const double det = dot(e1, cross(e2, e3));
    const Vec3 g[3] = {scale(cross(e2, e3), 1.0 / det), scale(cross(e3, e1), 1.0 / det),
                       scale(cross(e1, e2), 1.0 / det)};
    for (int e = 0; e < 3; ++e)
      for (int x = 0; x < 3; ++x) grad[c * 9 + e * 3 + x] = (float)g[e][x];
    const double volume = std::fabs(det) / 6.0;
    for (int f = 0; f < 4; ++f) {
      const Vec3 a = v[kFace2Nodes[f][0]], b = v[kFace2Nodes[f][1]], cc = v[kFace2Nodes[f][2]];
      Vec3 nrm = cross(sub(b, a), sub(cc, a));
      const double area = 0.5 * norm(nrm);
      Vec3 t1 = sub(b, a);
      Vec3 t2 = cross(nrm, t1);
      nrm = scale(nrm, 1.0 / norm(nrm));
      t1 = scale(t1, 1.0 / norm(t1));
      t2 = scale(t2, 1.0 / norm(t2));
      Mat9 qgl, qgn, T, Ti;
      faceGodunov(m, c, f, qgl, qgn);
      rotation(nrm, t1, t2, T, Ti);
      const double fs = -2.0 * area / (6.0 * volume);
      const bool dr = m.ftype[c * 4 + f] == 1;
      for (int side = 0; side < 2; ++side) {
        const Mat9& qg = side == 0 ? qgl : qgn;
        const double s = side == 0 && dr ? 0.0 : fs;
        float* out = (side == 0 ? wplus : wminus).data() + (c * 4 + f) * 54;
        // G(k, l) = sum_q Qgod(k, q) C_0(q, l): C_0(6, 0) = -1, C_0(7, 3) = C_0(8, 5) = -1/2
        double G[9][6] = {};
        for (int k = 0; k < 9; ++k) {
          G[k][0] = -qg[k * 9 + 6];
          G[k][3] = -0.5 * qg[k * 9 + 7];
          G[k][5] = -0.5 * qg[k * 9 + 8];
        }
        for (int i = 0; i < 9; ++i)
          for (int j = 0; j < 6; ++j) {
            double acc = 0;
            for (int k = 0; k < 9; ++k) {
              double t = 0;
              for (int l = 0; l < 6; ++l) t += G[k][l] * T[j * 9 + l];
              acc += Ti[k * 9 + i] * t;
            }
            out[i + 9 * j] = (float)(s * acc);
          }
      }
    }
  }
}

double cflTimestep(const HostMesh& m, int order, double cfl) {
  std::vector<double> dt;
  cellTimesteps(m, order, cfl, dt);
  double best = 1e300;
  for (double v : dt) best = std::min(best, v);
  return best;
}

void cellTimesteps(const HostMesh& m, int order, double cfl, std::vector<double>& dt) {
  dt.assign(m.n, 0.0);
  for (int64_t c = 0; c < m.n; ++c) {
    Vec3 x[4];
    for (int k = 0; k < 4; ++k) x[k] = {m.coords[c * 12 + k * 3], m.coords[c * 12 + k * 3 + 1], m.coords[c * 12 + k * 3 + 2]};
    const double alpha = dot(sub(x[1], x[0]), cross(sub(x[2], x[0]), sub(x[3], x[0])));
    const double areas = norm(cross(sub(x[1], x[0]), sub(x[2], x[0]))) + norm(cross(sub(x[1], x[0]), sub(x[3], x[0]))) +
                         norm(cross(sub(x[2], x[0]), sub(x[3], x[0]))) + norm(cross(sub(x[2], x[1]), sub(x[3], x[1])));
    const double insphere = std::fabs(alpha) / areas;
    const double rho = m.material[c * 3], mu = m.material[c * 3 + 1], lam = m.material[c * 3 + 2];
    const double vp = std::sqrt((lam + 2 * mu) / rho);
    dt[c] = cfl * 2.0 * insphere / (vp * (2 * order - 1));
  }
}

void permuteCells(HostMesh& m, const std::vector<int64_t>& order) {
  const int64_t n = m.n;
  if ((int64_t)order.size() != n) throw std::invalid_argument("permutation size");
  std::vector<int64_t> topo(n * 4);
  std::vector<double> coords(n * 12), material(n * 3);
  std::vector<int8_t> bc(m.bc.empty() ? 0 : n * 4);
  for (int64_t i = 0; i < n; ++i) {
    const int64_t o = order[i];
    for (int k = 0; k < 4; ++k) topo[i * 4 + k] = m.topo[o * 4 + k];
    for (int k = 0; k < 12; ++k) coords[i * 12 + k] = m.coords[o * 12 + k];
    for (int k = 0; k < 3; ++k) material[i * 3 + k] = m.material[o * 3 + k];
    if (!bc.empty())
      for (int k = 0; k < 4; ++k) bc[i * 4 + k] = m.bc[o * 4 + k];  // face numbering stays with the cell
  }
  m.topo.swap(topo);
  m.coords.swap(coords);
  m.material.swap(material);
  m.bc.swap(bc);
  computeFaceRelations(m);
}

void seedDofs(int64_t n, int order, uint64_t seed, std::vector<float>& dofs) {
  const int b = numBasis(order), bp = paddedBasis(order);
  dofs.assign(n * 9 * bp, 0.f);
  Rng rng(seed ^ 0x5DEECE66Dull);
  for (int64_t c = 0; c < n; ++c)
    for (int q = 0; q < 9; ++q)
      for (int k = 0; k < b; ++k) dofs[(c * 9 + q) * bp + k] = static_cast<float>(rng.uniform(-1.0, 1.0));
}

}  // namespace sei

namespace sei {

void buildPlanarFault(HostMesh& m, double xf, double h, HostFault& F) {
  const int kMissing[4] = {3, 2, 1, 0};  // FACE2MISSINGNODE
  F = HostFault();
  std::vector<int> drCount(m.n, 0);
  for (int64_t c = 0; c < m.n; ++c)
    for (int f = 0; f < 4; ++f) {
      bool on = true;
      for (int k = 0; k < 3; ++k) on = on && std::fabs(m.coords[c * 12 + kFace2Nodes[f][k] * 3] - xf) < 1e-9 * h;
      if (!on || m.coords[c * 12 + kMissing[f] * 3] >= xf) continue;  // plus side: rest of the cell at x < xf
      const int32_t d = m.nbr[c * 4 + f];
      if (d < 0) continue;
      const int j = m.side[c * 4 + f];
      F.plus_cell.push_back((int32_t)c);
      F.plus_side.push_back((uint8_t)f);
      F.minus_cell.push_back(d);
      F.minus_side.push_back((uint8_t)j);
      F.rel.push_back((uint8_t)(m.orient[c * 4 + f] + 1));
      m.ftype[c * 4 + f] = 1;
      m.ftype[(int64_t)d * 4 + j] = 1;
      ++drCount[c];
      ++drCount[d];
    }
  F.nf = (int64_t)F.plus_cell.size();
  for (int64_t c = 0; c < m.n; ++c)
    if (drCount[c] > 1) throw std::invalid_argument("a cell with more than one dynamic-rupture face is not supported");
  if (F.nf == 0) throw std::invalid_argument("fault plane has no faces (plane index outside the mesh?)");
}

void ingestMesh(const sei_mesh& p, HostMesh& m, HostFault& F) {
  const int kMissing[4] = {3, 2, 1, 0};  // FACE2MISSINGNODE
  if (p.nvertices <= 0 || p.ncells <= 0 || !p.geometry || !p.connect || !p.material)
    throw std::invalid_argument("mesh needs vertices, cells, connectivity and materials");
  if (p.ncells > (int64_t)1 << 30) throw std::invalid_argument("more than 2^30 cells");
  if (p.boundary && (p.boundary_format < SEI_BOUNDARY_I32 || p.boundary_format > SEI_BOUNDARY_I32X4))
    throw std::invalid_argument("unknown boundary format");
  if (p.fault_ref_method != SEI_FAULT_REF_POINT && p.fault_ref_method != SEI_FAULT_REF_NORMAL)
    throw std::invalid_argument("unknown fault reference method");
  const int64_t n = p.ncells;
  m = HostMesh();
  F = HostFault();
  m.n = n;
  m.topo.resize(n * 4);
  m.coords.resize(n * 12);
  m.material.assign(p.material, p.material + n * 3);
  for (int64_t c = 0; c < n; ++c) {
    const double r = m.material[c * 3], mu = m.material[c * 3 + 1], lam = m.material[c * 3 + 2];
    if (!(r > 0) || !(mu > 0) || !(lam + 2 * mu > 0) || !std::isfinite(r) || !std::isfinite(mu) || !std::isfinite(lam))
      throw std::invalid_argument("cell " + std::to_string(c) + ": material needs rho > 0, mu > 0, lambda + 2 mu > 0");
    for (int k = 0; k < 4; ++k) {
      const int64_t v = p.connect[c * 4 + k];
      if (v < 0 || v >= p.nvertices) throw std::invalid_argument("cell " + std::to_string(c) + ": vertex id out of range");
      int64_t t = v;
      if (p.identify) {
        t = p.identify[v];
        if (t < 0 || t >= p.nvertices) throw std::invalid_argument("identify: vertex id out of range");
      }
      m.topo[c * 4 + k] = t;
      for (int x = 0; x < 3; ++x) {
        const double q = p.geometry[v * 3 + x];
        if (!std::isfinite(q)) throw std::invalid_argument("non-finite vertex coordinate");
        m.coords[c * 12 + k * 3 + x] = q;
      }
    }
    // positive orientation (PUML convention): det [v1 - v0, v2 - v0, v3 - v0] > 0
    const double* w = &m.coords[c * 12];
    const Vec3 e1{w[3] - w[0], w[4] - w[1], w[5] - w[2]}, e2{w[6] - w[0], w[7] - w[1], w[8] - w[2]},
        e3{w[9] - w[0], w[10] - w[1], w[11] - w[2]};
    if (!(dot(e1, cross(e2, e3)) > 0))
      throw std::invalid_argument("cell " + std::to_string(c) + " is not positively oriented");
  }
  computeFaceRelations(m);
  // boundary condition of every face (docs/puml-mesh-format.rst; the default face map of
  // src/Initializer/FaceMap.cpp:100-110: 0, 6 regular; 1 free surface; 2 gravity free surface;
  // 3 and above 64 dynamic rupture; 4 Dirichlet; 5 outflow; 7 analytical)
  auto code = [&](int64_t c, int f) -> int64_t {
    if (!p.boundary) return 0;
    switch (p.boundary_format) {
      case SEI_BOUNDARY_I32: return (int64_t)((static_cast<const uint32_t*>(p.boundary)[c] >> (8 * f)) & 0xFFu);
      case SEI_BOUNDARY_I64: return (int64_t)((static_cast<const uint64_t*>(p.boundary)[c] >> (16 * f)) & 0xFFFFu);
      default: return (int64_t)static_cast<const int32_t*>(p.boundary)[c * 4 + f];
    }
  };
  m.bc.assign(n * 4, 0);
  std::vector<char> dr(n * 4, 0);
  for (int64_t c = 0; c < n; ++c)
    for (int f = 0; f < 4; ++f) {
      const int64_t b = code(c, f);
      const int32_t d = m.nbr[c * 4 + f];
      const std::string where = "cell " + std::to_string(c) + " face " + std::to_string(f);
      if (b == 0 || b == 6) {
        if (d < 0) throw std::invalid_argument(where + ": regular face without a neighbour");
      } else if (b == 3 || b > 64) {
        if (d < 0) throw std::invalid_argument(where + ": dynamic-rupture face without a neighbour");
        dr[c * 4 + f] = 1;
        dr[(int64_t)d * 4 + m.side[c * 4 + f]] = 1;
      } else if (b == 1 || b == 5) {
        if (d >= 0) throw std::invalid_argument(where + ": boundary condition on a face with a neighbour");
        m.bc[c * 4 + f] = (int8_t)b;
      } else if (b == 2 || b == 4 || b == 7) {
        throw std::domain_error(where + ": boundary condition " + std::to_string(b) +
                                " (gravity free surface, Dirichlet or analytical) is not supported");
      } else {
        throw std::invalid_argument(where + ": boundary condition " + std::to_string(b) + " is not defined");
      }
    }
  for (int64_t c = 0; c < n; ++c)
    for (int f = 0; f < 4; ++f)
      if (m.nbr[c * 4 + f] < 0 && m.bc[c * 4 + f] == 0)
        throw std::invalid_argument("cell " + std::to_string(c) + " face " + std::to_string(f) +
                                    ": mesh boundary without a boundary condition");
  // fault faces, each from its plus side: the cell on the reference point's side of the face
  // (Point), or whose outward face normal points along the reference vector (Normal)
  // (src/Geometry/MeshReader.cpp:150-170)
  const Vec3 ref{p.fault_ref[0], p.fault_ref[1], p.fault_ref[2]};
  auto isPlus = [&](int64_t c, int f, bool& onPlane) {
    const double* w = &m.coords[c * 12];
    auto vx = [&](int k) { return Vec3{w[k * 3], w[k * 3 + 1], w[k * 3 + 2]}; };
    const Vec3 a = vx(kFace2Nodes[f][0]);
    const Vec3 nrm = cross(sub(vx(kFace2Nodes[f][1]), a), sub(vx(kFace2Nodes[f][2]), a));
    const double s = p.fault_ref_method == SEI_FAULT_REF_POINT
                         ? dot(sub(ref, a), nrm) * dot(sub(vx(kMissing[f]), a), nrm)
                         : dot(ref, nrm);
    onPlane = s == 0.0;
    return s > 0.0;
  };
  for (int64_t c = 0; c < n; ++c)
    for (int f = 0; f < 4; ++f) {
      if (!dr[c * 4 + f]) continue;
      m.ftype[c * 4 + f] = 1;
      bool onPlane = false;
      if (!isPlus(c, f, onPlane)) {
        if (onPlane)
          throw std::invalid_argument("fault reference decides no side of the face of cell " + std::to_string(c));
        continue;
      }
      const int32_t d = m.nbr[c * 4 + f];
      const int j = m.side[c * 4 + f];
      bool dPlane = false;
      if (isPlus(d, j, dPlane))
        throw std::invalid_argument("fault reference puts both cells of a face on the plus side (cell " +
                                    std::to_string(c) + ")");
      F.plus_cell.push_back((int32_t)c);
      F.plus_side.push_back((uint8_t)f);
      F.minus_cell.push_back(d);
      F.minus_side.push_back((uint8_t)j);
      F.rel.push_back((uint8_t)(m.orient[c * 4 + f] + 1));
    }
  F.nf = (int64_t)F.plus_cell.size();
  if (F.nf > 0) faultFaceData(m, F);
}

void faultFaceData(const HostMesh& m, HostFault& F) {
  F.tinvt.assign(F.nf * 81, 0.f);
  F.fsp.assign(F.nf * 81, 0.f);
  F.fsm.assign(F.nf * 81, 0.f);
  F.imp.assign(F.nf * 8, 0.0);
  auto cellVec = [&](int64_t c, int k) {
    return Vec3{m.coords[c * 12 + k * 3], m.coords[c * 12 + k * 3 + 1], m.coords[c * 12 + k * 3 + 2]};
  };
  auto areaVolume = [&](int64_t c, int side, double& area, double& vol) {
    const Vec3 a = cellVec(c, kFace2Nodes[side][0]), b = cellVec(c, kFace2Nodes[side][1]), cc = cellVec(c, kFace2Nodes[side][2]);
    area = 0.5 * norm(cross(sub(b, a), sub(cc, a)));
    vol = std::fabs(dot(sub(cellVec(c, 3), cellVec(c, 0)), cross(sub(cellVec(c, 1), cellVec(c, 0)), sub(cellVec(c, 2), cellVec(c, 0))))) / 6.0;
  };
  for (int64_t f = 0; f < F.nf; ++f) {
    const int64_t pc = F.plus_cell[f], mc = F.minus_cell[f];
    const int ps = F.plus_side[f], ms = F.minus_side[f];
    const Vec3 a = cellVec(pc, kFace2Nodes[ps][0]), b = cellVec(pc, kFace2Nodes[ps][1]), cc = cellVec(pc, kFace2Nodes[ps][2]);
    Vec3 nrm = cross(sub(b, a), sub(cc, a));
    nrm = scale(nrm, 1.0 / norm(nrm));
    Vec3 t1 = sub(b, a);
    t1 = scale(t1, 1.0 / norm(t1));
    const Vec3 t2 = cross(nrm, t1);
    Mat9 T, Ti;
    rotation(nrm, t1, t2, T, Ti);
    for (int i = 0; i < 9; ++i)
      for (int j = 0; j < 9; ++j) F.tinvt[f * 81 + i + 9 * j] = (float)Ti[j * 9 + i];  // TinvT(i, j) = Tinv(j, i)
    double ap, vp, am, vm;
    areaVolume(pc, ps, ap, vp);
    areaVolume(mc, ms, am, vm);
    const double* mp = &m.material[pc * 3];
    const double* mm = &m.material[mc * 3];
    Mat9 atp, atm;
    coefficientMatrixT(mp[0], mp[1], mp[2], 0, atp);
    coefficientMatrixT(mm[0], mm[1], mm[2], 0, atm);
    const double sp = -2.0 * ap / (6.0 * vp), sm = 2.0 * am / (6.0 * vm);
    // fluxSolver(q, p) = scale * sum_k A^T(q, k) T(p, k)  (dynamic_rupture.py rotateFluxMatrix)
    for (int q = 0; q < 9; ++q)
      for (int p = 0; p < 9; ++p) {
        double vpv = 0, vmv = 0;
        for (int k = 0; k < 9; ++k) {
          vpv += atp[q * 9 + k] * T[p * 9 + k];
          vmv += atm[q * 9 + k] * T[p * 9 + k];
        }
        F.fsp[f * 81 + q + 9 * p] = (float)(sp * vpv);
        F.fsm[f * 81 + q + 9 * p] = (float)(sm * vmv);
      }
    const double zp = std::sqrt(mp[0] * (mp[2] + 2 * mp[1])), zs = std::sqrt(mp[0] * mp[1]);
    const double zpn = std::sqrt(mm[0] * (mm[2] + 2 * mm[1])), zsn = std::sqrt(mm[0] * mm[1]);
    double* im = &F.imp[f * 8];
    im[0] = zp;
    im[1] = zs;
    im[2] = zpn;
    im[3] = zsn;
    im[4] = 1.0 / (1.0 / zp + 1.0 / zpn);
    im[5] = 1.0 / (1.0 / zs + 1.0 / zsn);
    im[6] = 1.0 / zs + 1.0 / zsn;
  }
}

double fvwSteadyState(double v, double a, double b, double f0, double v0, double muw, double vw) {
  double lowv = f0 - (b - a) * std::log(v / v0);
  lowv = lowv > 0 ? lowv : 0.0;
  const double r = v / vw;
  const double fss = muw + (lowv - muw) / std::pow(1.0 + std::pow(r, 8.0), 0.125);
  const double c = fss / a;
  const double sign = c >= 0 ? 1.0 : -1.0, ac = std::fabs(c);
  return a * (ac + std::log(v0 / v * 2 / 2 * -sign * std::expm1(-2 * ac)));
}

void gaussLegendre01(int n, double* x, double* w) {
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5)), dp = 1;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1, p1 = z;
      for (int k = 2; k <= n; ++k) {
        const double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) p1 = z, p0 = 1;
      dp = n * (z * p1 - p0) / (z * z - 1);
      const double dz = p1 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[n - 1 - i] = 0.5 * (z + 1);  // ascending on [0, 1]
    w[n - 1 - i] = 1.0 / ((1 - z * z) * dp * dp);
  }
}

}  // namespace sei
