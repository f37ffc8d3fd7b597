// Seeded synthetic BAT trajectories (linear chain of n_atoms atoms:
// nb = n_atoms-1 bonds, na = n_atoms-2 angles, nd = n_atoms-3 dihedrals,
// matching PARENT's nBonds = nDih+2, nAngles = nDih+1, PARENT.cpp:298-299).
//
// Every value is a pure function of (seed, DOF, frame) through a counter-based
// hash, so host threads and device threads produce the same distribution in
// any order. The per-frame sampling code is shared by the host path
// (pg_synth_host) and the device kernel (pg_synth_device); the two use their
// own libm (glibc vs CUDA), so they agree in distribution, not bit-for-bit.
//
// Model:
//   latents  L_k(f) = phi L_k(f-1) + sqrt(1-phi^2) eta,  phi = 0.95, L_k(0) ~ N(0,1)
//   mixing   m_g(f) = sum_k w_gk L_k(f),  w_gk ~ N(0, 0.3)
//   bond     0.15 + 0.005 (e + m)/sqrt(1 + |w|^2)       (+0.02 in the second state of a bimodal bond)
//   angle    1.91 + VM(0, 40) + 0.158 m/sqrt(1 + |w|^2), clipped to [1e-6, pi - 1e-6]
//   dihedral mu_mode + VM(0, kappa_mode) + 0.3 m/sqrt(1 + |w|^2), wrapped to [0, 2 pi)
//            1-3 modes, mu ~ U(-pi, pi], kappa ~ U[2, 20]; the mode is drawn per frame
//            from the mode weights, or follows a two-state Markov chain for the
//            bimodal-switching fraction.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "../../include/parent_gb300.h"
#include "pg_internal.h"

namespace pg {
namespace synth {

#define HD __host__ __device__ __forceinline__

HD uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
HD uint64_t hash4(uint64_t seed, uint64_t stream, uint64_t a, uint64_t b) {
    return mix64(mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) ^ a) ^ (b * 0x8CB92BA72F3D8DD7ull));
}
// uniform in (0, 1), 53-bit
HD double unif(uint64_t h) { return ((double)(h >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

HD double normal(uint64_t seed, uint64_t stream, uint64_t a, uint64_t b) {
    const double u1 = unif(hash4(seed, stream, a, 2 * b));
    const double u2 = unif(hash4(seed, stream, a, 2 * b + 1));
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// von Mises(0, kappa) by Best & Fisher (1979), Applied Statistics 28:152-157.
// The rejection loop is capped at 64 rounds (acceptance is > 65% per round).
HD double vonmises(double kappa, uint64_t seed, uint64_t stream, uint64_t a, uint64_t b) {
    const double pi = 3.141592653589793;
    const double tau = 1.0 + sqrt(1.0 + 4.0 * kappa * kappa);
    const double rho = (tau - sqrt(2.0 * tau)) / (2.0 * kappa);
    const double r = (1.0 + rho * rho) / (2.0 * rho);
    double f = 0.0;
    uint64_t base = hash4(seed, stream, a, b);
    for (int it = 0; it < 64; it++) {
        const double u1 = unif(mix64(base + 3 * it));
        const double u2 = unif(mix64(base + 3 * it + 1));
        const double z = cos(pi * u1);
        f = (1.0 + r * z) / (r + z);
        const double c = kappa * (r - f);
        if (c * (2.0 - c) - u2 > 0.0) break;
        if (log(c / u2) + 1.0 - c >= 0.0) break;
    }
    if (f > 1.0) f = 1.0;
    if (f < -1.0) f = -1.0;
    const double u3 = unif(mix64(base + 191));
    const double th = acos(f);
    return u3 < 0.5 ? -th : th;
}

// Stream ids.
enum { S_LAT = 1, S_W = 2, S_BOND = 3, S_BIMOD = 4, S_ANG = 5, S_DMODE = 6, S_DVAL = 7, S_DPAR = 8, S_SW = 9 };

struct DofModel {
    double wnorm;          // 1/sqrt(1+|w|^2)
    int nmodes;            // dihedrals
    double mu[3], kappa[3], cw[3];  // cumulative mode weights
    int bimodal;           // Markov-switching DOF
};

HD void dof_model(uint64_t seed, int g, int type, int n_latents, double frac_bi_dih,
                  double frac_bi_bond, DofModel &m, float *w /* n_latents */) {
    double s = 0.0;
    for (int k = 0; k < n_latents; k++) {
        double wk = 0.3 * normal(seed, S_W, (uint64_t)g, (uint64_t)k);
        w[k] = (float)wk;
        s += (double)w[k] * (double)w[k];
    }
    m.wnorm = 1.0 / sqrt(1.0 + s);
    const double ub = unif(hash4(seed, S_BIMOD, (uint64_t)g, 0));
    m.bimodal = 0;
    m.nmodes = 1;
    if (type == TB) m.bimodal = ub < frac_bi_bond;
    if (type == TD) {
        m.bimodal = ub < frac_bi_dih;
        m.nmodes = m.bimodal ? 2 : 1 + (int)(3.0 * unif(hash4(seed, S_DPAR, (uint64_t)g, 0)));
        if (m.nmodes > 3) m.nmodes = 3;
        double tot = 0.0;
        for (int q = 0; q < 3; q++) {
            m.mu[q] = -3.141592653589793 + 6.283185307179586 * unif(hash4(seed, S_DPAR, (uint64_t)g, 1 + q));
            m.kappa[q] = 2.0 + 18.0 * unif(hash4(seed, S_DPAR, (uint64_t)g, 4 + q));
            const double wq = q < m.nmodes ? 0.2 + 0.8 * unif(hash4(seed, S_DPAR, (uint64_t)g, 7 + q)) : 0.0;
            tot += wq;
            m.cw[q] = tot;
        }
        for (int q = 0; q < 3; q++) m.cw[q] /= tot;
    }
}

// State of a Markov-switching DOF at frame f: parity of the number of switch
// times <= f in the DOF's sorted switch list.
HD int markov_state(const int *sw, int nsw, int f) {
    int lo = 0, hi = nsw;  // first index with sw[idx] > f
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (sw[mid] <= f) lo = mid + 1; else hi = mid;
    }
    return lo & 1;
}

HD double sample_value(uint64_t seed, int g, int type, int f, const DofModel &m, double mixv,
                       int state) {
    const double pi = 3.141592653589793, twopi = 6.283185307179586;
    if (type == TB) {
        const double e = normal(seed, S_BOND, (uint64_t)g, (uint64_t)f);
        double b = 0.15 + 0.005 * (e + mixv) * m.wnorm;
        if (m.bimodal && state) b += 0.02;
        return b;
    }
    if (type == TA) {
        double a = 1.91 + vonmises(40.0, seed, S_ANG, (uint64_t)g, (uint64_t)f) + 0.158 * mixv * m.wnorm;
        if (a < 1e-6) a = 1e-6;
        if (a > pi - 1e-6) a = pi - 1e-6;
        return a;
    }
    int q;
    if (m.bimodal) {
        q = state;
    } else {
        const double u = unif(hash4(seed, S_DMODE, (uint64_t)g, (uint64_t)f));
        q = u < m.cw[0] ? 0 : (u < m.cw[1] ? 1 : 2);
        if (q >= m.nmodes) q = m.nmodes - 1;
    }
    double d = m.mu[q] + vonmises(m.kappa[q], seed, S_DVAL, (uint64_t)g, (uint64_t)f) + 0.3 * mixv * m.wnorm;
    d = d - twopi * floor(d / twopi);
    if (!(d >= 0.0) || d >= twopi) d = 0.0;
    return d;
}

// Stores v as the output type; an FP32 dihedral that rounds up to >= 2 pi is
// wrapped to 0 (float(2 pi) > 2 pi would put it outside the reference's
// 100-bin shift histogram).
HD void store(void *base, int64_t idx, double v, int prec, int type) {
    if (prec) {
        ((double *)base)[idx] = v;
    } else {
        float fv = (float)v;
        if (type == TD && (double)fv >= 6.283185307179586) fv = 0.0f;
        if (type == TA && (double)fv >= 3.141592653589793) fv = nextafterf(3.14159265f, 0.0f);
        ((float *)base)[idx] = fv;
    }
}

// Host-side set-up shared by both paths: AR(1) latents [n_latents][F] and the
// sorted switch-frame lists of the Markov-switching DOFs (geometric gaps with
// per-frame switch probability p_switch).
static void prepare(const pg_synth_spec &sp, std::vector<float> &lat, std::vector<int> &sw,
                    std::vector<int> &sw_off) {
    const int F = sp.n_frames, L = sp.n_latents;
    const int nb = sp.n_atoms - 1, na = sp.n_atoms - 2, nd = sp.n_atoms - 3, D = nb + na + nd;
    lat.assign((size_t)L * F, 0.0f);
    const double phi = 0.95, sq = sqrt(1.0 - phi * phi);
    for (int k = 0; k < L; k++) {
        double v = normal(sp.seed, S_LAT, (uint64_t)k, 0);
        lat[(size_t)k * F] = (float)v;
        for (int f = 1; f < F; f++) {
            v = phi * v + sq * normal(sp.seed, S_LAT, (uint64_t)k, (uint64_t)f);
            lat[(size_t)k * F + f] = (float)v;
        }
    }
    sw.clear();
    sw_off.assign((size_t)D + 1, 0);
    std::vector<float> w(L > 0 ? L : 1);
    for (int g = 0; g < D; g++) {
        sw_off[g] = (int)sw.size();
        const int type = dof_type(g, nb, na);
        DofModel m{};
        dof_model(sp.seed, g, type, L, sp.frac_bimodal_dih, sp.frac_bimodal_bond, m, w.data());
        if (!m.bimodal || !(sp.p_switch > 0.0)) continue;
        // geometric gaps: next switch after floor(log(u)/log(1-p)) + 1 frames
        const double lq = log1p(-sp.p_switch);
        double pos = 0.0;
        for (uint64_t it = 0;; it++) {
            const double u = unif(hash4(sp.seed, S_SW, (uint64_t)g, it));
            pos += floor(log(u) / lq) + 1.0;
            if (pos >= (double)F) break;
            sw.push_back((int)pos);
        }
    }
    sw_off[D] = (int)sw.size();
}

__global__ void synth_kernel(pg_synth_spec sp, void *bonds, void *angles, void *dihedrals,
                             int64_t ld, const float *lat, const int *sw, const int *sw_off) {
    __shared__ DofModel m;
    __shared__ float w[32];
    const int nb = sp.n_atoms - 1, na = sp.n_atoms - 2;
    const int g = blockIdx.y;
    const int type = dof_type(g, nb, na);
    if (threadIdx.x == 0) dof_model(sp.seed, g, type, sp.n_latents, sp.frac_bimodal_dih,
                                    sp.frac_bimodal_bond, m, w);
    __syncthreads();
    void *base = type == TB ? bonds : (type == TA ? angles : dihedrals);
    const int local = g - (type == TB ? 0 : (type == TA ? nb : nb + na));
    const int *s = sw + sw_off[g];
    const int nsw = sw_off[g + 1] - sw_off[g];
    const int f0 = blockIdx.x * 4096;
    for (int f = f0 + threadIdx.x; f < f0 + 4096 && f < sp.n_frames; f += blockDim.x) {
        double mixv = 0.0;
        for (int k = 0; k < sp.n_latents; k++) mixv += (double)w[k] * (double)lat[(size_t)k * sp.n_frames + f];
        const int state = m.bimodal ? markov_state(s, nsw, f) : 0;
        store(base, (int64_t)local * ld + f, sample_value(sp.seed, g, type, f, m, mixv, state),
              sp.double_prec, type);
    }
}

}  // namespace synth

void set_global_error(const char *msg);

bool synth_spec_ok(const pg_synth_spec *sp) {
    return sp && sp->n_atoms >= 3 && sp->n_frames >= 1 && sp->n_latents >= 0 && sp->n_latents <= 32 &&
           (sp->double_prec == 0 || sp->double_prec == 1) && sp->p_switch >= 0.0 && sp->p_switch < 1.0;
}

// Device path: latents and switch lists are prepared on the host, uploaded
// into `scratch` (caller-provided device memory of synth_scratch_bytes), then
// one block per (4096-frame chunk, DOF) samples the values.
size_t synth_scratch_bytes(const pg_synth_spec *sp, size_t *lat_bytes, size_t *sw_bytes,
                           std::vector<float> &lat, std::vector<int> &sw, std::vector<int> &sw_off) {
    synth::prepare(*sp, lat, sw, sw_off);
    *lat_bytes = (lat.size() * sizeof(float) + 255) / 256 * 256;
    *sw_bytes = ((sw.size() + sw_off.size()) * sizeof(int) + 255) / 256 * 256;
    return *lat_bytes + *sw_bytes;
}

cudaError_t launch_synth_dev(const pg_synth_spec *sp, void *b, void *a, void *d, int64_t ld,
                             const float *lat, const int *sw, const int *sw_off, cudaStream_t st) {
    const int D = 3 * sp->n_atoms - 6;
    dim3 grid((sp->n_frames + 4095) / 4096, D);
    synth::synth_kernel<<<grid, 256, 0, st>>>(*sp, b, a, d, ld, lat, sw, sw_off);
    return cudaGetLastError();
}

}  // namespace pg

extern "C" PG_API int pg_synth_host(const pg_synth_spec *sp, void *bonds, void *angles,
                                    void *dihedrals, int64_t ld, int n_threads) {
    using namespace pg;
    using namespace pg::synth;
    if (!synth_spec_ok(sp) || !bonds || !angles || (!dihedrals && sp->n_atoms > 3) || ld < sp->n_frames) {
        set_global_error("pg_synth_host: invalid spec (n_atoms >= 3, n_frames >= 1, 0 <= n_latents <= 32, "
                         "double_prec 0/1, 0 <= p_switch < 1) or null/short buffers");
        return PG_ERR_ARG;
    }
    std::vector<float> lat;
    std::vector<int> sw, sw_off;
    prepare(*sp, lat, sw, sw_off);
    const int nb = sp->n_atoms - 1, na = sp->n_atoms - 2, nd = sp->n_atoms - 3, D = nb + na + nd;
    const int F = sp->n_frames, L = sp->n_latents;
    if (n_threads <= 0) n_threads = (int)std::max(1u, std::thread::hardware_concurrency());
    n_threads = std::min(n_threads, D);
    auto work = [&](int t) {
        std::vector<float> w(L > 0 ? L : 1);
        for (int g = t; g < D; g += n_threads) {
            const int type = dof_type(g, nb, na);
            DofModel m{};
            dof_model(sp->seed, g, type, L, sp->frac_bimodal_dih, sp->frac_bimodal_bond, m, w.data());
            void *base = type == TB ? bonds : (type == TA ? angles : dihedrals);
            const int local = g - (type == TB ? 0 : (type == TA ? nb : nb + na));
            const int *s = sw.data() + sw_off[g];
            const int nsw = sw_off[g + 1] - sw_off[g];
            for (int f = 0; f < F; f++) {
                double mixv = 0.0;
                for (int k = 0; k < L; k++) mixv += (double)w[k] * (double)lat[(size_t)k * F + f];
                const int state = m.bimodal ? markov_state(s, nsw, f) : 0;
                store(base, (int64_t)local * ld + f, sample_value(sp->seed, g, type, f, m, mixv, state),
                      sp->double_prec, type);
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 1; t < n_threads; t++) th.emplace_back(work, t);
    work(0);
    for (auto &x : th) x.join();
    return PG_OK;
}
