// synth.cpp -- seeded synthetic catchment generator for benchmarks and tests.
//
// Produces the static inputs Wflow would read from a staticmaps netCDF for a square raster:
// a fractal DEM (diamond-square), a depression-free surface (priority-flood with an epsilon
// gradient, one corner outlet as the only pit), a D8 local drain direction in PCRaster codes
// 1-9 consistent with Wflow's PCR_DIR (Wflow/src/utils.jl:3-13, x = first index), the
// downstream index of every cell, flow length/width (Wflow/src/utils.jl:418-449), slope and
// upstream cell counts. Cell order is Julia's column-major order of an (x, y) raster:
// index = y * nx + x. Only integer arithmetic, + - * / and sqrt are used so that the same
// seed gives the same domain on every IEEE-754 host.
#include <cstdint>
#include <cstring>
#include <queue>
#include <vector>
#include <cmath>

namespace {

struct SplitMix {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    // uniform in [-1, 1)
    double sym() { return (double)(next() >> 11) * 0x1p-52 - 1.0; }
};

}  // namespace

extern "C" {

// Returns 0 on success, -1 on bad arguments.
//   hurst in (0, 1]; scale_ratio = 2^-hurst must be given by the caller (no pow here).
int32_t wf_synth_dem_d8(int32_t nx, int32_t ny, uint64_t seed, double scale_ratio, double zmax,
                        double cell_size, double min_slope, double tilt, double* dem, uint8_t* ldd,
                        int32_t* downstream, double* slope, int64_t* upstream_cells,
                        double* flow_length, double* flow_width) {
    if (nx < 1 || ny < 1 || !(scale_ratio > 0.0) || !(cell_size > 0.0)) return -1;
    // ---- diamond-square on a (2^k + 1) square grid
    int size = 2;
    while (size + 1 < nx || size + 1 < ny) size *= 2;
    const int S = size + 1;
    std::vector<double> h((size_t)S * S, 0.0);
    auto H = [&](int x, int y) -> double& { return h[(size_t)y * S + x]; };
    SplitMix rng{seed * 0x2545F4914F6CDD1DULL + 1};
    H(0, 0) = rng.sym();
    H(size, 0) = rng.sym();
    H(0, size) = rng.sym();
    H(size, size) = rng.sym();
    double amp = 1.0;
    for (int step = size; step > 1; step /= 2) {
        int half = step / 2;
        amp *= scale_ratio;
        for (int y = half; y < S; y += step)
            for (int x = half; x < S; x += step) {
                double avg = (H(x - half, y - half) + H(x + half, y - half) + H(x - half, y + half) +
                              H(x + half, y + half)) * 0.25;
                H(x, y) = avg + amp * rng.sym();
            }
        for (int y = 0; y < S; y += half) {
            for (int x = ((y / half) % 2 == 0) ? half : 0; x < S; x += step) {
                double sum = 0.0;
                int cnt = 0;
                if (x - half >= 0) { sum += H(x - half, y); ++cnt; }
                if (x + half < S) { sum += H(x + half, y); ++cnt; }
                if (y - half >= 0) { sum += H(x, y - half); ++cnt; }
                if (y + half < S) { sum += H(x, y + half); ++cnt; }
                H(x, y) = sum / cnt + amp * rng.sym();
            }
        }
    }
    // crop, add the regional plane dipping to the outlet corner (relative weight `tilt` of the
    // fractal relief) and rescale to [0, zmax]
    const int64_t n = (int64_t)nx * ny;
    double flo = 1e300, fhi = -1e300;
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            double v = H(x, y);
            flo = v < flo ? v : flo;
            fhi = v > fhi ? v : fhi;
        }
    const double relief = fhi - flo > 0.0 ? fhi - flo : 1.0;
    const double diag_len = (double)(nx - 1) + (double)(ny - 1) > 0.0 ? (double)(nx - 1) + (double)(ny - 1) : 1.0;
    double lo = 1e300, hi = -1e300;
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            double v = H(x, y) + tilt * relief * ((double)x + (double)y) / diag_len;
            dem[(int64_t)y * nx + x] = v;
            lo = v < lo ? v : lo;
            hi = v > hi ? v : hi;
        }
    double span = hi - lo > 0.0 ? hi - lo : 1.0;
    for (int64_t i = 0; i < n; ++i) dem[i] = (dem[i] - lo) / span * zmax;
    // ---- priority-flood + epsilon from the single outlet at (0, 0)
    const double eps = 1e-5;
    std::vector<uint8_t> seen(n, 0);
    struct Item {
        double z;
        uint64_t seq;
        int64_t i;
        bool operator<(const Item& o) const { return z > o.z || (z == o.z && seq > o.seq); }
    };
    std::priority_queue<Item> pq;
    uint64_t seq = 0;
    dem[0] = -1.0;  // outlet below every other cell
    seen[0] = 1;
    pq.push({dem[0], seq++, 0});
    static const int DX[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
    static const int DY[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
    while (!pq.empty()) {
        Item it = pq.top();
        pq.pop();
        int x = (int)(it.i % nx), y = (int)(it.i / nx);
        for (int k = 0; k < 8; ++k) {
            int xx = x + DX[k], yy = y + DY[k];
            if (xx < 0 || yy < 0 || xx >= nx || yy >= ny) continue;
            int64_t j = (int64_t)yy * nx + xx;
            if (seen[j]) continue;
            seen[j] = 1;
            double zmin = dem[it.i] + eps;
            if (dem[j] < zmin) dem[j] = zmin;
            pq.push({dem[j], seq++, j});
        }
    }
    // ---- D8 steepest descent, PCRaster codes: code = (dy + 1) * 3 + (dx + 1) + 1
    const double diag = cell_size * std::sqrt(2.0);
    for (int64_t i = 0; i < n; ++i) {
        int x = (int)(i % nx), y = (int)(i / nx);
        int best = -1;
        double best_s = 0.0;
        for (int k = 0; k < 8; ++k) {
            int xx = x + DX[k], yy = y + DY[k];
            if (xx < 0 || yy < 0 || xx >= nx || yy >= ny) continue;
            int64_t j = (int64_t)yy * nx + xx;
            double dist = (DX[k] != 0 && DY[k] != 0) ? diag : cell_size;
            double s = (dem[i] - dem[j]) / dist;
            if (s > best_s) {
                best_s = s;
                best = k;
            }
        }
        if (i == 0 || best < 0) {
            ldd[i] = 5;
            downstream[i] = -1;
            slope[i] = min_slope;
            flow_length[i] = diag;  // hypot(x_length, y_length) for LDD 5
            flow_width[i] = (cell_size * cell_size) / diag;
        } else {
            int dx = DX[best], dy = DY[best];
            ldd[i] = (uint8_t)((dy + 1) * 3 + (dx + 1) + 1);
            downstream[i] = (int32_t)((int64_t)(y + dy) * nx + (x + dx));
            bool straight_y = (ldd[i] == 2 || ldd[i] == 8), straight_x = (ldd[i] == 4 || ldd[i] == 6);
            flow_length[i] = straight_y || straight_x ? cell_size : diag;
            flow_width[i] = straight_y || straight_x ? cell_size : (cell_size * cell_size) / diag;
            double s = (dem[i] - dem[downstream[i]]) / flow_length[i];
            slope[i] = s > min_slope ? s : min_slope;
        }
    }
    dem[0] = dem[0] < 0.0 ? 0.0 : dem[0];
    // ---- upstream cell counts (including the cell itself), Kahn order from the sources
    std::vector<int32_t> indeg(n, 0);
    for (int64_t i = 0; i < n; ++i)
        if (downstream[i] >= 0) indeg[downstream[i]]++;
    std::vector<int64_t> order;
    order.reserve(n);
    for (int64_t i = 0; i < n; ++i) {
        upstream_cells[i] = 1;
        if (indeg[i] == 0) order.push_back(i);
    }
    for (size_t q = 0; q < order.size(); ++q) {
        int64_t v = order[q];
        int32_t d = downstream[v];
        if (d >= 0) {
            upstream_cells[d] += upstream_cells[v];
            if (--indeg[d] == 0) order.push_back(d);
        }
    }
    return (int64_t)order.size() == n ? 0 : -2;
}

}  // extern "C"
