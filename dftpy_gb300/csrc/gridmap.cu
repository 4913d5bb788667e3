// Fourier interpolation of a real field between two grids of one cell
// (grid_map_data / grid_map_index, src/dftpy/utils/utils.py:50-128, as
// field2distrib uses it at utils.py:218-285): R2C on the source grid, one
// gather of the source half spectrum into the destination half spectrum, C2R
// on the destination grid, with an optional floor on the result.
#include "common.cuh"

namespace ofdft {
namespace {

// grid_map_index along one full axis: the source index whose coefficient lands
// on destination index I, or -1.  Finer destination: source indices above
// ns/2 move up by nd - ns; coarser destination: destination indices above
// nd/2 read from ns - nd further up.
__device__ inline int map_axis(int I, int nd, int ns) {
    if (nd >= ns) {
        if (I <= ns / 2) return I;
        const int t = I - (nd - ns);
        return (t > ns / 2 && t < ns) ? t : -1;
    }
    return I <= nd / 2 ? I : I + (ns - nd);
}

template <typename C>
__device__ inline C gather(const C* src, const Geo& s, const Geo& d, int I, int J, int K) {
    C z;
    z.x = 0;
    z.y = 0;
    const int i = map_axis(I, d.n0, s.n0), j = map_axis(J, d.n1, s.n1);
    if (i < 0 || j < 0 || K >= s.n2h) return z;
    return src[((long long)i * s.n1 + j) * s.n2h + K];
}

// On the k2 = 0 and k2 = n2/2 planes the destination C2R reads only the
// Hermitian part of the data (numpy's irfftn drops the imaginary part of those
// bins after the inverse transforms over axes 0 and 1), so the gathered plane
// is replaced by (F(G) + conj F(-G)) / 2 there.
template <typename C>
__global__ void k_grid_map(const C* __restrict__ src, Geo s, C* __restrict__ dst, Geo d, double scale) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < d.Nc; idx += stride) {
        const int K = (int)(idx % d.n2h);
        const long long t = idx / d.n2h;
        const int J = (int)(t % d.n1), I = (int)(t / d.n1);
        C v = gather(src, s, d, I, J, K);
        double re = (double)v.x, im = (double)v.y;
        if (K == 0 || (d.n2 % 2 == 0 && K == d.n2 / 2)) {
            const int Ip = I == 0 ? 0 : d.n0 - I, Jp = J == 0 ? 0 : d.n1 - J;
            const C p = gather(src, s, d, Ip, Jp, K);
            re = 0.5 * (re + (double)p.x);
            im = 0.5 * (im - (double)p.y);
        }
        dst[idx].x = re * scale;
        dst[idx].y = im * scale;
    }
}

template <typename T>
__global__ void k_floor(T* x, long long n, T lo) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
        if (x[i] < lo) x[i] = lo;
}

template <typename T>
void map_t(ofdft_grid* src, ofdft_grid* dst, const void* in, void* out, double floor_value, cudaStream_t st) {
    using C = typename Cplx<T>::type;
    C* sG = (C*)src->scratch.get("map_src", src->cplx_bytes());
    C* dG = (C*)dst->scratch.get("map_dst", dst->cplx_bytes());
    src->exec_r2c(in, sG, 1, st);
    // rfftn * dV_src on the source, irfftn / dV_dst on the destination
    const double scale = src->dV / (dst->dV * (double)dst->N);
    const int nb = blocks_for(dst->Nc, 256, dst->sms * 8);
    k_grid_map<C><<<nb, 256, 0, st>>>(sG, src->geo, dG, dst->geo, scale);
    OFDFT_LAUNCH_CHECK();
    dst->exec_c2r(dG, out, 1, st);
    if (std::isfinite(floor_value)) {
        const int fb = blocks_for(dst->N, 256, dst->sms * 8);
        k_floor<T><<<fb, 256, 0, st>>>((T*)out, dst->N, (T)floor_value);
        OFDFT_LAUNCH_CHECK();
    }
}

}  // namespace
}  // namespace ofdft

using namespace ofdft;

extern "C" int ofdft_grid_map(ofdft_grid* src, ofdft_grid* dst, const void* in, void* out, double floor_value,
                              ofdft_stream s) {
    return guard([&] {
        OFDFT_REQUIRE(src && dst && in && out, "ofdft_grid_map: null argument");
        OFDFT_REQUIRE(src->prec == dst->prec, "ofdft_grid_map: the grids differ in precision");
        OFDFT_REQUIRE(std::fabs(src->volume - dst->volume) <= 1e-10 * src->volume,
                      "ofdft_grid_map: the grids belong to different cells");
        bool up = true, down = true;
        for (int d = 0; d < 3; ++d) {
            up = up && dst->nr[d] >= src->nr[d];
            down = down && dst->nr[d] <= src->nr[d];
        }
        OFDFT_REQUIRE(up || down, "ofdft_grid_map: the destination grid must be finer or coarser on every axis");
        OFDFT_REQUIRE(in != out, "ofdft_grid_map: out aliases in");
        if (src->prec == OFDFT_F64)
            map_t<double>(src, dst, in, out, floor_value, (cudaStream_t)s);
        else
            map_t<float>(src, dst, in, out, floor_value, (cudaStream_t)s);
    });
}
