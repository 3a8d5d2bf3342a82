// Fused finite-volume assembly: RHS F(x) and Jacobian values in one pass
// per cell, straight into the fixed-width stencil CSR.
//
// One thread owns one cell.  It builds that cell's atoms -- the coefficients
// of every (d1, d2, offset) coupling -- in registers, applies the boundary
// program for the faces the cell touches, and then either contracts the
// atom with the state (RHS) or writes it out as CSR values (Jacobian).
//
// The arithmetic follows the reference term by term and in the same order
// (transiflow/Discretization.py, BoundaryConditions.py, CrsMatrix.py), and
// this file is compiled with -fmad=false, so the results agree with the
// reference bit for bit.  All divisions are precomputed per axis on the host
// (the rD/rH/w0/w1 metric fields), so the kernel only multiplies and adds.

#include <type_traits>
#include <utility>

#include "tf_common.cuh"

namespace tf {

template <int I>
using ic = std::integral_constant<int, I>;

template <class F, int... Is>
__device__ __forceinline__ void static_for_impl(F &&f, std::integer_sequence<int, Is...>) {
    (f(ic<Is>{}), ...);
}
template <int N, class F>
__device__ __forceinline__ void static_for(F &&f) {
    static_for_impl(f, std::make_integer_sequence<int, N>{});
}

// ---------------------------------------------------------------------------
// Layouts: the Jacobian atom uses the full stencil template; the Picard
// (F) atom never holds velocity-velocity cross couplings, so it uses the
// template without them.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr bool in_template_F(int DIM, int DOF, int d1, int d2, int ox, int oy, int oz) {
    return in_template(DIM, DOF, d1, d2, ox, oy, oz) && !(d1 < DIM && d2 < DIM && d1 != d2);
}

template <int DIM, int DOF, bool FONLY>
struct LayoutK {
    int slot[DOF][DOF][27];
    int width;
    __host__ __device__ constexpr LayoutK() : slot{}, width(0) {
        int p = 0;
        for (int d1 = 0; d1 < DOF; ++d1) {
            for (int d2 = 0; d2 < DOF; ++d2)
                for (int o = 0; o < 27; ++o) slot[d1][d2][o] = -1;
            for (int oz = 0; oz < 3; ++oz)
                for (int oy = 0; oy < 3; ++oy)
                    for (int ox = 0; ox < 3; ++ox)
                        for (int d2 = 0; d2 < DOF; ++d2) {
                            bool in = FONLY ? in_template_F(DIM, DOF, d1, d2, ox, oy, oz)
                                            : in_template(DIM, DOF, d1, d2, ox, oy, oz);
                            if (in) slot[d1][d2][off_index(ox, oy, oz)] = p++;
                        }
        }
        width = p;
    }
};

template <int DIM, int DOF, bool FONLY>
constexpr LayoutK<DIM, DOF, FONLY> kLayout{};

template <int DIM, int DOF, bool FONLY>
struct Atom {
    static constexpr int W = kLayout<DIM, DOF, FONLY>.width;
    template <int d1, int d2, int o>
    static constexpr int S = kLayout<DIM, DOF, FONLY>.slot[d1][d2][o];
    double v[W];

    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int s = 0; s < W; ++s) v[s] = 0.0;
    }
    template <int d1, int d2, int o>
    __device__ __forceinline__ void sub(double x) {
        constexpr int s = S<d1, d2, o>;
        static_assert(s >= 0, "coupling outside the stencil template");
        v[s] = v[s] - x;
    }
    template <int d1, int d2, int o>
    __device__ __forceinline__ void set(double x) {
        constexpr int s = S<d1, d2, o>;
        static_assert(s >= 0, "coupling outside the stencil template");
        v[s] = x;
    }
};

// offset index with axis a at value va and axis b at value vb, others 1
__host__ __device__ constexpr int off2(int a, int va, int b, int vb) {
    int o[3] = {1, 1, 1};
    o[a] = va;
    o[b] = vb;
    return off_index(o[0], o[1], o[2]);
}
__host__ __device__ constexpr int off1(int a, int va) {
    int o[3] = {1, 1, 1};
    o[a] = va;
    return off_index(o[0], o[1], o[2]);
}
// offset index with axis a at value va and the other two axes (in increasing
// axis order) taking q % 3 and q / 3
__host__ __device__ constexpr int off_q(int a, int va, int q) {
    int o[3] = {0, 0, 0};
    int b1 = a == 0 ? 1 : 0;
    int b2 = a == 2 ? 1 : 2;
    o[a] = va;
    o[b1] = q % 3;
    o[b2] = q / 3;
    return off_index(o[0], o[1], o[2]);
}
constexpr int OC = 13;   // centre offset (1,1,1)

// ---------------------------------------------------------------------------
// Per-cell context: metrics and padded-state reads
// ---------------------------------------------------------------------------
struct Ctx {
    const tf_problem &p;
    const double *__restrict__ st;
    int i, j, k;

    __device__ __forceinline__ double m(int axis, int field, int idx) const {
        return __ldg(p.d_metric + (axis * TF_METRIC_FIELDS + field) * p.metric_stride + idx);
    }
    // utils.create_padded_state_mtx (utils.py:62-133) read at cell (ci, cj, ck)
    __device__ __forceinline__ double s(int ci, int cj, int ck, int d) const {
        if (p.nz == 1) ck = 0;   // z periodic with a single cell
        if (ci < 0 || ci >= p.nx || cj < 0 || cj >= p.ny || ck < 0 || ck >= p.nz) return 0.0;
        if (d == 0 && ci == p.nx - 1) return 0.0;
        if (d == 1 && cj == p.ny - 1) return 0.0;
        if (d == 2 && p.nz > 1 && ck == p.nz - 1) return 0.0;
        return __ldg(st + d + p.dof * (ci + p.nx * (cj + p.ny * ck)));
    }
    // average_x/y/z (Discretization.py:1178-1209) at a face index
    __device__ __forceinline__ double avx(int d, int fi, int cj, int ck) const {
        return 0.5 * s(fi - 1, cj, ck, d) + 0.5 * s(fi, cj, ck, d);
    }
    __device__ __forceinline__ double avy(int d, int ci, int fj, int ck) const {
        return 0.5 * s(ci, fj - 1, ck, d) + 0.5 * s(ci, fj, ck, d);
    }
    __device__ __forceinline__ double avz(int d, int ci, int cj, int fk) const {
        return 0.5 * s(ci, cj, fk - 1, d) + 0.5 * s(ci, cj, fk, d);
    }
    // weighted_average_x/y/z (Discretization.py:1211-1266); ci/cj/ck is the
    // cell whose spacing weights the two values
    __device__ __forceinline__ double wx(int d, int ci, int cj, int ck) const {
        return m(0, M_W0, ci) * s(ci, cj, ck, d) + m(0, M_W1, ci) * s(ci + 1, cj, ck, d);
    }
    __device__ __forceinline__ double wy(int d, int ci, int cj, int ck) const {
        return m(1, M_W0, cj) * s(ci, cj, ck, d) + m(1, M_W1, cj) * s(ci, cj + 1, ck, d);
    }
    __device__ __forceinline__ double wz(int d, int ci, int cj, int ck) const {
        return m(2, M_W0, ck) * s(ci, cj, ck, d) + m(2, M_W1, ck) * s(ci, cj, ck + 1, d);
    }
};

// ---------------------------------------------------------------------------
// Nonlinear part (Discretization.nonlinear_part, Discretization.py:319-365)
// ---------------------------------------------------------------------------

// u_u_x / v_v_y / w_w_z: identical updates of the F and J atoms
template <int var, int ax, bool WJ, class AF, class AJ>
__device__ __forceinline__ void self_conv(AF &F, AJ &J, double a2, double Alo, double Ahi) {
    const double a1 = -a2;
    const double t1 = a1 * Alo * 1.0 / 2.0;
    const double t2 = a2 * Ahi * 1.0 / 2.0;
    F.template sub<var, var, off1(ax, 0)>(t1);
    F.template sub<var, var, OC>(t1);
    F.template sub<var, var, OC>(t2);
    F.template sub<var, var, off1(ax, 2)>(t2);
    if constexpr (WJ) {
        J.template sub<var, var, off1(ax, 0)>(t1);
        J.template sub<var, var, OC>(t1);
        J.template sub<var, var, OC>(t2);
        J.template sub<var, var, off1(ax, 2)>(t2);
    }
}

// u_v_x-type term: Picard part on (row,row) along axr, linearisation on
// (row,col) over axr x axc (e.g. Discretization.py:1281-1295)
template <int row, int col, int axr, int axc, bool WJ, class AF, class AJ>
__device__ __forceinline__ void cross(AF &F, AJ &J, double b1, double tw0, double tw1,
                                      double ac0, double ac1, double w0, double w1) {
    const double b0 = -b1;
    const double tF0 = b0 * tw0 * 1.0 / 2.0;
    const double tF1 = b1 * tw1 * 1.0 / 2.0;
    F.template sub<row, row, off1(axr, 0)>(tF0);
    F.template sub<row, row, OC>(tF0);
    F.template sub<row, row, OC>(tF1);
    F.template sub<row, row, off1(axr, 2)>(tF1);
    if constexpr (WJ) {
        const double p0 = b0 * ac0;
        const double p1 = b1 * ac1;
        J.template sub<row, col, off2(axr, 0, axc, 1)>(p0 * w0);
        J.template sub<row, col, off2(axr, 0, axc, 2)>(p0 * w1);
        J.template sub<row, col, off2(axr, 1, axc, 1)>(p1 * w0);
        J.template sub<row, col, off2(axr, 1, axc, 2)>(p1 * w1);
    }
}

// u_C_x / v_C_y / w_C_z for the temperature (Discretization.py:1313-1459)
template <int var, int ax, bool WJ, class AF, class AJ>
__device__ __forceinline__ void scalar_conv(AF &F, AJ &J, double q1, double Ulo, double Uhi,
                                            double Clo, double Chi) {
    const double q0 = -q1;
    const double t0 = q0 * Ulo * 1.0 / 2.0;
    const double t1 = q1 * Uhi * 1.0 / 2.0;
    F.template sub<var, var, off1(ax, 0)>(t0);
    F.template sub<var, var, OC>(t0);
    F.template sub<var, var, OC>(t1);
    F.template sub<var, var, off1(ax, 2)>(t1);
    if constexpr (WJ) {
        J.template sub<var, ax, off1(ax, 0)>(q0 * Clo);
        J.template sub<var, ax, OC>(q1 * Chi);
    }
}

template <int DIM, int DOF, bool WJ, class AF, class AJ>
__device__ __forceinline__ void nonlinear(const Ctx &c, AF &F, AJ &J) {
    const int i = c.i, j = c.j, k = c.k;
    const double Dx = c.m(0, M_D, i), Dy = c.m(1, M_D, j), Dz = c.m(2, M_D, k);
    const double Hpx = c.m(0, M_HP, i), Hpy = c.m(1, M_HP, j), Hpz = c.m(2, M_HP, k);
    // u_u_x
    self_conv<0, 0, WJ>(F, J, Dy * Dz, c.avx(0, i, j, k), c.avx(0, i + 1, j, k));
    // u_v_x (v row, J wrt u)
    cross<1, 0, 0, 1, WJ>(F, J, Hpy * Dz, c.wy(0, i - 1, j, k), c.wy(0, i, j, k),
                          c.avx(1, i, j, k), c.avx(1, i + 1, j, k),
                          c.m(1, M_W0, j), c.m(1, M_W1, j));
    // v_u_y (u row, J wrt v)
    cross<0, 1, 1, 0, WJ>(F, J, Hpx * Dz, c.wx(1, i, j - 1, k), c.wx(1, i, j, k),
                          c.avy(0, i, j, k), c.avy(0, i, j + 1, k),
                          c.m(0, M_W0, i), c.m(0, M_W1, i));
    // v_v_y
    self_conv<1, 1, WJ>(F, J, Dx * Dz, c.avy(1, i, j, k), c.avy(1, i, j + 1, k));
    if constexpr (DIM > 2) {
        // u_w_x (w row, J wrt u)
        cross<2, 0, 0, 2, WJ>(F, J, Hpz * Dy, c.wz(0, i - 1, j, k), c.wz(0, i, j, k),
                              c.avx(2, i, j, k), c.avx(2, i + 1, j, k),
                              c.m(2, M_W0, k), c.m(2, M_W1, k));
        // v_w_y (w row, J wrt v)
        cross<2, 1, 1, 2, WJ>(F, J, Hpz * Dx, c.wz(1, i, j - 1, k), c.wz(1, i, j, k),
                              c.avy(2, i, j, k), c.avy(2, i, j + 1, k),
                              c.m(2, M_W0, k), c.m(2, M_W1, k));
        // w_u_z (u row, J wrt w)
        cross<0, 2, 2, 0, WJ>(F, J, Hpx * Dy, c.wx(2, i, j, k - 1), c.wx(2, i, j, k),
                              c.avz(0, i, j, k), c.avz(0, i, j, k + 1),
                              c.m(0, M_W0, i), c.m(0, M_W1, i));
        // w_v_z (v row, J wrt w)
        cross<1, 2, 2, 1, WJ>(F, J, Hpy * Dx, c.wy(2, i, j, k - 1), c.wy(2, i, j, k),
                              c.avz(1, i, j, k), c.avz(1, i, j, k + 1),
                              c.m(1, M_W0, j), c.m(1, M_W1, j));
        // w_w_z
        self_conv<2, 2, WJ>(F, J, Dy * Dx, c.avz(2, i, j, k), c.avz(2, i, j, k + 1));
    }
    if constexpr (DOF > DIM + 1) {
        constexpr int T = DIM + 1;
        scalar_conv<T, 0, WJ>(F, J, Dy * Dz, c.s(i - 1, j, k, 0), c.s(i, j, k, 0),
                              c.avx(T, i, j, k), c.avx(T, i + 1, j, k));
        scalar_conv<T, 1, WJ>(F, J, Dx * Dz, c.s(i, j - 1, k, 1), c.s(i, j, k, 1),
                              c.avy(T, i, j, k), c.avy(T, i, j + 1, k));
        if constexpr (DIM > 2)
            scalar_conv<T, 2, WJ>(F, J, Dy * Dx, c.s(i, j, k - 1, 2), c.s(i, j, k, 2),
                                  c.avz(T, i, j, k), c.avz(T, i, j, k + 1));
    }
    if constexpr (DOF > DIM + 2) {
        // u_S_x, v_S_y (Discretization.py:1331-1400)
        constexpr int Sv = DIM + 2;
        scalar_conv<Sv, 0, WJ>(F, J, Dy * Dz, c.s(i - 1, j, k, 0), c.s(i, j, k, 0),
                               c.avx(Sv, i, j, k), c.avx(Sv, i + 1, j, k));
        scalar_conv<Sv, 1, WJ>(F, J, Dx * Dz, c.s(i, j - 1, k, 1), c.s(i, j, k, 1),
                               c.avy(Sv, i, j, k), c.avy(Sv, i, j + 1, k));
        if constexpr (DIM > 2)
            scalar_conv<Sv, 2, WJ>(F, J, Dy * Dx, c.s(i, j, k - 1, 2), c.s(i, j, k, 2),
                                   c.avz(Sv, i, j, k), c.avz(Sv, i, j, k + 1));
    }
}

// ---------------------------------------------------------------------------
// Linear part (Discretization._linear_part_2D/3D, Discretization.py:229-317)
// added slot by slot: A[s] = A[s] + lin[s].
// ---------------------------------------------------------------------------
struct Diff {   // one second-difference primitive: values at offsets 0,1,2
    double a0, a1, a2;
};
__device__ __forceinline__ Diff second(double rlo, double rhi, double w1, double w2) {
    Diff d;
    d.a0 = rlo * w1 * w2;
    d.a2 = rhi * w1 * w2;
    d.a1 = -d.a0 - d.a2;
    return d;
}

template <int DIM, int DOF, class A>
__device__ __forceinline__ void add_linear(const Ctx &c, A &at) {
    const int i = c.i, j = c.j, k = c.k;
    const double Dx = c.m(0, M_D, i), Dy = c.m(1, M_D, j), Dz = c.m(2, M_D, k);
    const double Hpx = c.m(0, M_HP, i), Hpy = c.m(1, M_HP, j), Hpz = c.m(2, M_HP, k);
    const double rDx = c.m(0, M_RD, i), rDy = c.m(1, M_RD, j), rDz = c.m(2, M_RD, k);
    const double rDpx = c.m(0, M_RDP, i), rDpy = c.m(1, M_RDP, j), rDpz = c.m(2, M_RDP, k);
    const double rHx = c.m(0, M_RH, i), rHy = c.m(1, M_RH, j), rHz = c.m(2, M_RH, k);
    const double rHpx = c.m(0, M_RHP, i), rHpy = c.m(1, M_RHP, j), rHpz = c.m(2, M_RHP, k);
    const double visc = c.p.visc;

    auto add = [&](auto D1, auto D2, auto O, double x) {
        constexpr int s = A::template S<decltype(D1)::value, decltype(D2)::value, decltype(O)::value>;
        static_assert(s >= 0, "linear term outside the stencil template");
        at.v[s] = at.v[s] + x;
    };
    // velocity diffusion: visc * (sum of the primitives) per slot; the centre
    // is the sum over axes in x, y, z order
    auto vel = [&](auto V, Diff dx, Diff dy, Diff dz) {
        add(V, V, ic<off1(0, 0)>{}, visc * dx.a0);
        add(V, V, ic<off1(0, 2)>{}, visc * dx.a2);
        add(V, V, ic<off1(1, 0)>{}, visc * dy.a0);
        add(V, V, ic<off1(1, 2)>{}, visc * dy.a2);
        if constexpr (DIM > 2) {
            add(V, V, ic<off1(2, 0)>{}, visc * dz.a0);
            add(V, V, ic<off1(2, 2)>{}, visc * dz.a2);
            add(V, V, ic<OC>{}, visc * (dx.a1 + dy.a1 + dz.a1));
        } else {
            add(V, V, ic<OC>{}, visc * (dx.a1 + dy.a1));
        }
    };
    Diff z0{0, 0, 0};
    vel(ic<0>{}, second(rDx, rDpx, Dy, Dz), second(rHy, rHpy, Hpx, Dz),
        DIM > 2 ? second(rHz, rHpz, Hpx, Dy) : z0);
    vel(ic<1>{}, second(rHx, rHpx, Hpy, Dz), second(rDy, rDpy, Dx, Dz),
        DIM > 2 ? second(rHz, rHpz, Hpy, Dx) : z0);
    if constexpr (DIM > 2)
        vel(ic<2>{}, second(rHx, rHpx, Hpz, Dy), second(rHy, rHpy, Hpz, Dx), second(rDz, rDpz, Dy, Dx));

    constexpr int P = DIM;
    // - (p_x + p_y + p_z): 0 - (-g) = g at offset 1, 0 - g = -g at offset 2
    const double gx = Dy * Dz, gy = Dx * Dz, gz = Dy * Dx;
    add(ic<0>{}, ic<P>{}, ic<off1(0, 1)>{}, 0.0 - (-gx));
    add(ic<0>{}, ic<P>{}, ic<off1(0, 2)>{}, 0.0 - gx);
    add(ic<1>{}, ic<P>{}, ic<off1(1, 1)>{}, 0.0 - (-gy));
    add(ic<1>{}, ic<P>{}, ic<off1(1, 2)>{}, 0.0 - gy);
    // + div
    add(ic<P>{}, ic<0>{}, ic<off1(0, 0)>{}, -gx);
    add(ic<P>{}, ic<0>{}, ic<off1(0, 1)>{}, gx);
    add(ic<P>{}, ic<1>{}, ic<off1(1, 0)>{}, -gy);
    add(ic<P>{}, ic<1>{}, ic<off1(1, 1)>{}, gy);
    if constexpr (DIM > 2) {
        add(ic<2>{}, ic<P>{}, ic<off1(2, 1)>{}, 0.0 - (-gz));
        add(ic<2>{}, ic<P>{}, ic<off1(2, 2)>{}, 0.0 - gz);
        add(ic<P>{}, ic<2>{}, ic<off1(2, 0)>{}, -gz);
        add(ic<P>{}, ic<2>{}, ic<off1(2, 1)>{}, gz);
    }
    if constexpr (DIM == 2 && A::template S<0, 1, 1 + 0 * 3 + 9> >= 0) {
        // - beta * coriolis (Discretization.py:253-255, 1086-1099): the
        // linear atom holds 0 - beta * c at these slots, no other linear term
        // (an F atom without these slots belongs to a problem without it)
        if (c.p.rossby != 0.0) {
            const double beta = c.p.rossby;
            const double *aux = c.p.d_aux;
            const double cv = (Hpy * Dx * Dz / 2) * aux[j];                 // v row, u column
            const double cu = (Hpx * Dy * Dz / 2) * aux[c.p.ny + j];        // u row, v column
            const double lv = 0.0 - beta * cv, lu = 0.0 - beta * cu;
            add(ic<1>{}, ic<0>{}, ic<0 + 3 * 1 + 9>{}, lv);
            add(ic<1>{}, ic<0>{}, ic<0 + 3 * 2 + 9>{}, lv);
            add(ic<1>{}, ic<0>{}, ic<1 + 3 * 1 + 9>{}, lv);
            add(ic<1>{}, ic<0>{}, ic<1 + 3 * 2 + 9>{}, lv);
            add(ic<0>{}, ic<1>{}, ic<1 + 3 * 0 + 9>{}, lu);
            add(ic<0>{}, ic<1>{}, ic<2 + 3 * 0 + 9>{}, lu);
            add(ic<0>{}, ic<1>{}, ic<1 + 3 * 1 + 9>{}, lu);
            add(ic<0>{}, ic<1>{}, ic<2 + 3 * 1 + 9>{}, lu);
        }
    }
    if constexpr (DOF > DIM + 1) {
        constexpr int T = DIM + 1;
        const double cond = c.p.cond;
        Diff tx = second(rHx, rHpx, Dy, Dz), ty = second(rHy, rHpy, Dx, Dz);
        add(ic<T>{}, ic<T>{}, ic<off1(0, 0)>{}, cond * tx.a0);
        add(ic<T>{}, ic<T>{}, ic<off1(0, 2)>{}, cond * tx.a2);
        add(ic<T>{}, ic<T>{}, ic<off1(1, 0)>{}, cond * ty.a0);
        add(ic<T>{}, ic<T>{}, ic<off1(1, 2)>{}, cond * ty.a2);
        if constexpr (DIM > 2) {
            Diff tz = second(rHz, rHpz, Dy, Dx);
            add(ic<T>{}, ic<T>{}, ic<off1(2, 0)>{}, cond * tz.a0);
            add(ic<T>{}, ic<T>{}, ic<off1(2, 2)>{}, cond * tz.a2);
            add(ic<T>{}, ic<T>{}, ic<OC>{}, cond * (tx.a1 + ty.a1 + tz.a1));
        } else {
            add(ic<T>{}, ic<T>{}, ic<OC>{}, cond * (tx.a1 + ty.a1));
        }
        // buoyancy: forward_average_T_y / _z (Discretization.py:1016-1057)
        if (c.p.buoy_row == 1) {
            const double fa = Hpy * Dx * Dz / 2.0;
            add(ic<1>{}, ic<T>{}, ic<off1(1, 1)>{}, fa);
            add(ic<1>{}, ic<T>{}, ic<off1(1, 2)>{}, fa);
        }
        if constexpr (DIM > 2) {
            if (c.p.buoy_row == 2) {
                const double fa = Hpz * Dy * Dx / 2.0;
                add(ic<2>{}, ic<T>{}, ic<off1(2, 1)>{}, fa);
                add(ic<2>{}, ic<T>{}, ic<off1(2, 2)>{}, fa);
            }
        }
        // Rayleigh-Benard perturbation: Bi/(Bi+1) * backward_average_{v_y,w_z}
        if (c.p.biot_row == 1) {
            const double ba = Hpy * Dx * Dz / 2.0;
            add(ic<T>{}, ic<1>{}, ic<off1(1, 0)>{}, c.p.biot * ba);
            add(ic<T>{}, ic<1>{}, ic<off1(1, 1)>{}, c.p.biot * ba);
        }
        if constexpr (DIM > 2) {
            if (c.p.biot_row == 2) {
                const double ba = Hpz * Dy * Dx / 2.0;
                add(ic<T>{}, ic<2>{}, ic<off1(2, 0)>{}, c.p.biot * ba);
                add(ic<T>{}, ic<2>{}, ic<off1(2, 1)>{}, c.p.biot * ba);
            }
        }
    }
    if constexpr (DOF > DIM + 2) {
        // salinity: sal * (S_xx + S_yy) - forward_average_S_y
        // (Discretization.py:260-263; the 2D layout is the only one compiled)
        static_assert(DIM == 2, "salinity is compiled for the 2D layout only");
        constexpr int Sv = DIM + 2;
        const double sal = c.p.sal;
        Diff sx = second(rHx, rHpx, Dy, Dz), sy = second(rHy, rHpy, Dx, Dz);
        add(ic<Sv>{}, ic<Sv>{}, ic<off1(0, 0)>{}, sal * sx.a0);
        add(ic<Sv>{}, ic<Sv>{}, ic<off1(0, 2)>{}, sal * sx.a2);
        add(ic<Sv>{}, ic<Sv>{}, ic<off1(1, 0)>{}, sal * sy.a0);
        add(ic<Sv>{}, ic<Sv>{}, ic<off1(1, 2)>{}, sal * sy.a2);
        add(ic<Sv>{}, ic<Sv>{}, ic<OC>{}, sal * (sx.a1 + sy.a1));
        const double fa = Hpy * Dx * Dz / 2.0;
        add(ic<1>{}, ic<Sv>{}, ic<off1(1, 1)>{}, 0.0 - fa);
        add(ic<1>{}, ic<Sv>{}, ic<off1(1, 2)>{}, 0.0 - fa);
    }
}

// ---------------------------------------------------------------------------
// Boundary program (BoundaryConditions.py:55-544), applied to one cell
// ---------------------------------------------------------------------------
// The forcing component zeroed by the east/north/top walls: u, v and -- as
// the reference does (BoundaryConditions.py:131, 221) -- v for the top wall.
__host__ __device__ constexpr int wall_frc_var(int a) { return a == 0 ? 0 : 1; }

template <int DIM, int DOF, bool FONLY, int a, bool high>
__device__ __forceinline__ void wall_op(Atom<DIM, DOF, FONLY> &A, double (&frc)[DOF], int sign) {
    using AT = Atom<DIM, DOF, FONLY>;
    constexpr int inner = high ? 2 : 0;
    if constexpr (!high) {
        // atom[0, ..., d2=a, off_a=0] = 0
        static_for<DOF>([&](auto D1) {
            static_for<9>([&](auto Q) {
                constexpr int s = AT::template S<decltype(D1)::value, a, off_q(a, 0, decltype(Q)::value)>;
                if constexpr (s >= 0) A.v[s] = 0.0;
            });
        });
    }
    // off_a = 1 (+/-)= off_a = outward
    static_for<DOF>([&](auto D1) {
        static_for<DOF>([&](auto D2) {
            static_for<9>([&](auto Q) {
                constexpr int d1 = decltype(D1)::value, d2 = decltype(D2)::value, q = decltype(Q)::value;
                constexpr int s1 = AT::template S<d1, d2, off_q(a, 1, q)>;
                constexpr int s2 = AT::template S<d1, d2, off_q(a, inner, q)>;
                static_assert(!(s2 >= 0 && s1 < 0), "boundary fold leaves the stencil template");
                if constexpr (s1 >= 0 && s2 >= 0) {
                    if (sign < 0) A.v[s1] = A.v[s1] - A.v[s2];
                    else A.v[s1] = A.v[s1] + A.v[s2];
                }
            });
        });
    });
    if constexpr (high) {
        // atom[b, ..., d2=a, off_a=1] = 0 ; atom[b, d1=a] = 0
        static_for<DOF>([&](auto D1) {
            static_for<9>([&](auto Q) {
                constexpr int s = AT::template S<decltype(D1)::value, a, off_q(a, 1, decltype(Q)::value)>;
                if constexpr (s >= 0) A.v[s] = 0.0;
            });
        });
        static_for<DOF>([&](auto D2) {
            static_for<27>([&](auto O) {
                constexpr int s = AT::template S<a, decltype(D2)::value, decltype(O)::value>;
                if constexpr (s >= 0) A.v[s] = 0.0;
            });
        });
    }
    // off_a = outward -> 0
    static_for<DOF>([&](auto D1) {
        static_for<DOF>([&](auto D2) {
            static_for<9>([&](auto Q) {
                constexpr int s = AT::template S<decltype(D1)::value, decltype(D2)::value,
                                                 off_q(a, inner, decltype(Q)::value)>;
                if constexpr (s >= 0) A.v[s] = 0.0;
            });
        });
    });
    if constexpr (high) {
        constexpr int sc = AT::template S<a, a, OC>;
        if constexpr (sc >= 0) A.v[sc] = -1.0;
        frc[wall_frc_var(a)] = 0.0;
    }
}

// atom[n-2, ..., d1=a, d2=a, off_a=2] = 0 (the "TODO" line of no_slip_*/free_slip_*)
template <int DIM, int DOF, bool FONLY, int a>
__device__ __forceinline__ void wall_second_op(Atom<DIM, DOF, FONLY> &A) {
    using AT = Atom<DIM, DOF, FONLY>;
    static_for<9>([&](auto Q) {
        constexpr int s = AT::template S<a, a, off_q(a, 2, decltype(Q)::value)>;
        if constexpr (s >= 0) A.v[s] = 0.0;
    });
}

template <int DIM, int DOF, bool FONLY, int a, bool high>
__device__ __forceinline__ void force_op(Atom<DIM, DOF, FONLY> &A, double (&frc)[DOF], int var,
                                         double fc, double ac, const double *prof = nullptr, int tcell = 0,
                                         int plen = 0) {
    using AT = Atom<DIM, DOF, FONLY>;
    constexpr int out = high ? 2 : 0;
    static_for<DOF>([&](auto V) {
        constexpr int vv = decltype(V)::value;
        if (vv != var) return;
        double acc = 0.0;
        static_for<9>([&](auto Q) {
            constexpr int q = decltype(Q)::value;
            constexpr int s = AT::template S<vv, vv, off_q(a, out, q)>;
            if constexpr (s >= 0) {
                if (prof) {
                    // a profile along the first tangential axis (2D: the
                    // second tangential offset is the centre)
                    int m = tcell + q % 3 - 1;
                    if (m < 0) m += plen;
                    acc = acc + A.v[s] * (q / 3 == 1 ? prof[m] : 0.0);
                } else {
                    acc = acc + A.v[s] * fc;
                }
            }
        });
        frc[vv] = frc[vv] + acc;
        static_for<DOF>([&](auto D1) {
            static_for<9>([&](auto Q) {
                constexpr int d1 = decltype(D1)::value, q = decltype(Q)::value;
                constexpr int s1 = AT::template S<d1, vv, off_q(a, 1, q)>;
                constexpr int s2 = AT::template S<d1, vv, off_q(a, out, q)>;
                if constexpr (s2 >= 0) {
                    static_assert(s1 >= 0, "forcing fold leaves the stencil template");
                    A.v[s1] = A.v[s1] + ac * A.v[s2];
                    A.v[s2] = 0.0;
                }
            });
        });
    });
}

// TF_BC_PIN (Discretization.py:690-702): entries coupling to var of cell
// (0,0,0), periodic neighbours included, become 0; cell 0's row var gets -1
// on its diagonal and no forcing.
template <int DIM, int DOF, bool FONLY>
__device__ __forceinline__ void pin_op(const Ctx &c, Atom<DIM, DOF, FONLY> &A, double (&frc)[DOF], int var) {
    using AT = Atom<DIM, DOF, FONLY>;
    const int nx = c.p.nx, ny = c.p.ny, nz = c.p.nz;
    static_for<DOF>([&](auto V) {
        constexpr int vv = decltype(V)::value;
        if (vv != var) return;
        static_for<DOF>([&](auto D1) {
            static_for<27>([&](auto O) {
                constexpr int d1 = decltype(D1)::value, o = decltype(O)::value;
                constexpr int s = AT::template S<d1, vv, o>;
                if constexpr (s >= 0) {
                    const bool hit = (c.i + o % 3 - 1 + nx) % nx == 0 && (c.j + (o / 3) % 3 - 1 + ny) % ny == 0 &&
                                     (c.k + o / 9 - 1 + nz) % nz == 0;
                    if (hit) A.v[s] = 0.0;
                }
            });
        });
        if (c.i == 0 && c.j == 0 && c.k == 0) {
            A.v[AT::template S<vv, vv, OC>] = -1.0;
            frc[vv] = 0.0;
        }
    });
}

template <int DIM, int DOF, bool FONLY>
__device__ __forceinline__ void boundaries(const Ctx &c, Atom<DIM, DOF, FONLY> &A, double (&frc)[DOF]) {
    const int idx[3] = {c.i, c.j, c.k};
    const int ext[3] = {c.p.nx, c.p.ny, c.p.nz};
    for (int t = 0; t < c.p.nops; ++t) {
        const tf_bc_op &op = c.p.ops[t];
        const int a = op.axis;
        const int n = ext[a];
        const int here = idx[a];
        const bool on = op.high ? here == n - 1 : here == 0;
        if (op.kind == TF_BC_WALL) {
            if (on) {
#define TF_WALL(AX, HI) wall_op<DIM, DOF, FONLY, AX, HI>(A, frc, op.var)
                if (a == 0) { if (op.high) TF_WALL(0, true); else TF_WALL(0, false); }
                else if (a == 1) { if (op.high) TF_WALL(1, true); else TF_WALL(1, false); }
                else if constexpr (DIM > 2) { if (op.high) TF_WALL(2, true); else TF_WALL(2, false); }
#undef TF_WALL
            } else if (op.high && here == ((n - 2) % n + n) % n) {
                if (a == 0) wall_second_op<DIM, DOF, FONLY, 0>(A);
                else if (a == 1) wall_second_op<DIM, DOF, FONLY, 1>(A);
                else if constexpr (DIM > 2) wall_second_op<DIM, DOF, FONLY, 2>(A);
            }
        } else if (op.kind == TF_BC_PIN) {
            pin_op<DIM, DOF, FONLY>(c, A, frc, op.var);
        } else if (op.kind == TF_BC_FORCE_PROFILE) {
            if constexpr (DIM == 2) {
                if (on) {
                    const double *prof = c.p.d_prof + (size_t)(int)op.fc * c.p.prof_len;
                    const int tcell = a == 0 ? c.j : c.i;
#define TF_FORCE(AX, HI) force_op<DIM, DOF, FONLY, AX, HI>(A, frc, op.var, 0.0, op.ac, prof, tcell, c.p.prof_len)
                    if (a == 0) { if (op.high) TF_FORCE(0, true); else TF_FORCE(0, false); }
                    else if (a == 1) { if (op.high) TF_FORCE(1, true); else TF_FORCE(1, false); }
#undef TF_FORCE
                }
            }
        } else if (on) {
#define TF_FORCE(AX, HI) force_op<DIM, DOF, FONLY, AX, HI>(A, frc, op.var, op.fc, op.ac)
            if (a == 0) { if (op.high) TF_FORCE(0, true); else TF_FORCE(0, false); }
            else if (a == 1) { if (op.high) TF_FORCE(1, true); else TF_FORCE(1, false); }
            else if constexpr (DIM > 2) { if (op.high) TF_FORCE(2, true); else TF_FORCE(2, false); }
#undef TF_FORCE
        }
    }
}

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
constexpr double DROP = 1e-14;   // CrsMatrix.compress threshold

// COR: a 2D problem with the Coriolis term, whose F atom then also holds the
// velocity-velocity couplings (the full template).
template <int DIM, int DOF, bool WF, bool WJ, bool COR = false>
__global__ void __launch_bounds__(128) assemble_kernel(const tf_problem p, const double *__restrict__ st,
                                                       double *__restrict__ rhs, double *__restrict__ jv) {
    const int ncell = p.nx * p.ny * p.nz;
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncell) return;
    Ctx c{p, st, cell % p.nx, (cell / p.nx) % p.ny, cell / (p.nx * p.ny)};

    Atom<DIM, DOF, !COR> F;
    Atom<DIM, DOF, false> J;
    F.zero();
    if constexpr (WJ) J.zero();
    if (p.nonlinear) nonlinear<DIM, DOF, WJ>(c, F, J);

    if constexpr (WJ) {
        using AF = Atom<DIM, DOF, !COR>;
        using AJ = Atom<DIM, DOF, false>;
        // atomJ += atomF (Discretization.py:363)
        static_for<DOF>([&](auto D1) {
            static_for<DOF>([&](auto D2) {
                static_for<27>([&](auto O) {
                    constexpr int d1 = decltype(D1)::value, d2 = decltype(D2)::value, o = decltype(O)::value;
                    constexpr int sf = AF::template S<d1, d2, o>;
                    constexpr int sj = AJ::template S<d1, d2, o>;
                    if constexpr (sf >= 0) J.v[sj] = J.v[sj] + F.v[sf];
                });
            });
        });
        add_linear<DIM, DOF>(c, J);
        double frcJ[DOF];
#pragma unroll
        for (int d = 0; d < DOF; ++d) frcJ[d] = 0.0;
        boundaries(c, J, frcJ);
        constexpr int W = AJ::W;
        double *out = jv + (size_t)cell * W;
#pragma unroll
        for (int s = 0; s < W; ++s) {
            const double x = J.v[s];
            out[s] = fabs(x) > DROP ? x : 0.0;
        }
    }
    if constexpr (WF) {
        using AF = Atom<DIM, DOF, !COR>;
        add_linear<DIM, DOF>(c, F);
        double frc[DOF];
#pragma unroll
        for (int d = 0; d < DOF; ++d) frc[d] = 0.0;
        if constexpr (DIM == 2) {
            // wind stress of the double gyre (Discretization.py:1101-1118):
            // u equation, every column but the east wall's
            if (p.wind != 0.0 && c.i < p.nx - 1) {
                const double *aux = p.d_aux;
                const double base = -(1 - p.asym) * aux[2 * p.ny + c.j] - p.asym * aux[3 * p.ny + c.j];
                frc[0] = base * (p.wind * c.m(0, M_HP, c.i) * c.m(1, M_D, c.j) * c.m(2, M_D, c.k));
            }
        }
        boundaries(c, F, frc);
        // assemble_rhs (Discretization.py:439-472): per row, the products in
        // (oz, oy, ox, d2) order, then + frc
        static_for<DOF>([&](auto D1) {
            constexpr int d1 = decltype(D1)::value;
            double acc = 0.0;
            static_for<27>([&](auto O) {
                constexpr int o = decltype(O)::value;
                static_for<DOF>([&](auto D2) {
                    constexpr int d2 = decltype(D2)::value;
                    constexpr int s = AF::template S<d1, d2, o>;
                    if constexpr (s >= 0)
                        acc = acc + F.v[s] * c.s(c.i + o % 3 - 1, c.j + (o / 3) % 3 - 1, c.k + o / 9 - 1, d2);
                });
            });
            rhs[(size_t)cell * DOF + d1] = acc + frc[d1];
        });
    }
}

template <int DIM, int DOF>
__global__ void pattern_kernel(const tf_problem p, int32_t *__restrict__ rowptr, int32_t *__restrict__ cols) {
    constexpr Layout<DIM, DOF> L{};
    constexpr int W = L.width();
    const int ncell = p.nx * p.ny * p.nz;
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncell) return;
    const int i = cell % p.nx, j = (cell / p.nx) % p.ny, k = cell / (p.nx * p.ny);
#pragma unroll
    for (int d1 = 0; d1 < DOF; ++d1) rowptr[cell * DOF + d1] = cell * W + L.rowoff[d1];
    if (cell == ncell - 1) rowptr[ncell * DOF] = ncell * W;
    static_for<DOF>([&](auto D1) {
        static_for<27>([&](auto O) {
            static_for<DOF>([&](auto D2) {
                constexpr int d1 = decltype(D1)::value, o = decltype(O)::value, d2 = decltype(D2)::value;
                constexpr int s = L.slot[d1][d2][o];
                if constexpr (s >= 0) {
                    int ci = i + o % 3 - 1, cj = j + (o / 3) % 3 - 1, ck = k + o / 9 - 1;
                    ci = ci < 0 ? 0 : (ci >= p.nx ? p.nx - 1 : ci);
                    cj = cj < 0 ? 0 : (cj >= p.ny ? p.ny - 1 : cj);
                    if (p.nz == 1) ck = 0;
                    ck = ck < 0 ? 0 : (ck >= p.nz ? p.nz - 1 : ck);
                    cols[(size_t)cell * W + s] = d2 + DOF * (ci + p.nx * (cj + p.ny * ck));
                }
            });
        });
    });
}

template <int DIM, int DOF>
__global__ void mass_kernel(const tf_problem p, double *__restrict__ diag) {
    const int ncell = p.nx * p.ny * p.nz;
    const int cell = blockIdx.x * blockDim.x + threadIdx.x;
    if (cell >= ncell) return;
    Ctx c{p, nullptr, cell % p.nx, (cell / p.nx) % p.ny, cell / (p.nx * p.ny)};
    const double Dx = c.m(0, M_D, c.i), Dy = c.m(1, M_D, c.j), Dz = c.m(2, M_D, c.k);
    const double Hpx = c.m(0, M_HP, c.i), Hpy = c.m(1, M_HP, c.j), Hpz = c.m(2, M_HP, c.k);
    double *o = diag + (size_t)cell * DOF;
    // mass_x/y/z/C, Discretization.py:1120-1176
    o[0] = Hpx * Dy * Dz;
    o[1] = Hpy * Dx * Dz;
    if constexpr (DIM == 3) o[2] = Hpz * Dy * Dx;
    o[DIM] = 0.0;
    if constexpr (DOF > DIM + 1) o[DIM + 1] = Dx * Dy * Dz;
    if constexpr (DOF > DIM + 2) o[DIM + 2] = Dx * Dy * Dz;
}

template <int DIM, int DOF>
static int stencil_layout(int *row_offset, int *slot) {
    constexpr Layout<DIM, DOF> L{};
    for (int d = 0; d <= DOF; ++d) row_offset[d] = L.rowoff[d];
    if (slot)
        for (int d1 = 0; d1 < DOF; ++d1)
            for (int d2 = 0; d2 < DOF; ++d2)
                for (int o = 0; o < 27; ++o) slot[(d1 * DOF + d2) * 27 + o] = L.slot[d1][d2][o];
    return TF_OK;
}

static int check_problem(const tf_problem *p) {
    if (!p || p->nx < 1 || p->ny < 1 || p->nz < 1 || !p->d_metric) return TF_ERR_ARG;
    if (p->nops < 0 || p->nops > TF_MAX_BC_OPS) return TF_ERR_ARG;
    if (p->metric_stride < p->nx || p->metric_stride < p->ny || p->metric_stride < p->nz) return TF_ERR_ARG;
    if ((int64_t)p->nx * p->ny * p->nz * 80 > INT32_MAX) return TF_ERR_SIZE;
    for (int t = 0; t < p->nops; ++t) {
        const tf_bc_op &op = p->ops[t];
        if (op.kind == TF_BC_FORCE_PROFILE) {
            if (p->dim != 2 || !p->d_prof || op.axis > 1) return TF_ERR_ARG;
            const int along = op.axis == 0 ? p->ny : p->nx;
            if (p->prof_len != along + 2 || !(op.fc >= 0 && op.fc < p->nprof)) return TF_ERR_ARG;
        }
        if ((op.kind == TF_BC_PIN || op.kind == TF_BC_FORCE || op.kind == TF_BC_FORCE_PROFILE) &&
            (op.var < 0 || op.var >= p->dof))
            return TF_ERR_ARG;
    }
    return TF_OK;
}

}  // namespace tf

using namespace tf;

extern "C" int tf_version(void) { return 1; }

extern "C" const char *tf_error_string(int code) {
    switch (code) {
        case TF_OK: return "ok";
        case TF_ERR_ARG: return "invalid argument";
        case TF_ERR_UNSUPPORTED: return "unsupported (dim, dof) combination";
        case TF_ERR_CUDA: return "CUDA error";
        case TF_ERR_SIZE: return "size exceeds a compiled-in limit";
        case TF_ERR_TIMEOUT: return "a device-side wait gave up";
        default: return "unknown error";
    }
}

extern "C" int tf_stencil_layout(int dim, int dof, int *row_offset, int *slot) {
    if (!row_offset) return TF_ERR_ARG;
#define TF_CALL(D, F) return stencil_layout<D, F>(row_offset, slot)
    TF_DISPATCH(dim, dof, TF_CALL);
#undef TF_CALL
}

extern "C" int tf_stencil_pattern(const tf_problem *p, int32_t *d_rowptr, int32_t *d_cols, tf_stream_t stream) {
    int e = check_problem(p);
    if (e) return e;
    if (!d_rowptr || !d_cols) return TF_ERR_ARG;
    const int ncell = p->nx * p->ny * p->nz;
    const int blocks = (ncell + 127) / 128;
#define TF_CALL(D, F) pattern_kernel<D, F><<<blocks, 128, 0, (cudaStream_t)stream>>>(*p, d_rowptr, d_cols); launched()
    TF_DISPATCH(p->dim, p->dof, TF_CALL);
#undef TF_CALL
    return cuda_status();
}

template <int D, int F, bool COR>
static void launch_assemble_c(int blocks, cudaStream_t s, const tf_problem &p, const double *st, double *rhs,
                              double *jv) {
    if (rhs && jv) assemble_kernel<D, F, true, true, COR><<<blocks, 128, 0, s>>>(p, st, rhs, jv);
    else if (rhs) assemble_kernel<D, F, true, false, COR><<<blocks, 128, 0, s>>>(p, st, rhs, jv);
    else assemble_kernel<D, F, false, true, COR><<<blocks, 128, 0, s>>>(p, st, rhs, jv);
}

template <int D, int F>
static void launch_assemble(bool cor, int blocks, cudaStream_t s, const tf_problem &p, const double *st,
                            double *rhs, double *jv) {
    if constexpr (D == 2) {
        if (cor) { launch_assemble_c<D, F, true>(blocks, s, p, st, rhs, jv); return; }
    }
    launch_assemble_c<D, F, false>(blocks, s, p, st, rhs, jv);
}

extern "C" int tf_assemble(const tf_problem *p, const double *d_state, double *d_rhs, double *d_jvals,
                           tf_stream_t stream) {
    int e = check_problem(p);
    if (e) return e;
    if (!d_state || (!d_rhs && !d_jvals)) return TF_ERR_ARG;
    const int ncell = p->nx * p->ny * p->nz;
    const int blocks = (ncell + 127) / 128;
    cudaStream_t s = (cudaStream_t)stream;
    if (p->rossby != 0.0 && p->dim != 2) return TF_ERR_UNSUPPORTED;
    if ((p->rossby != 0.0 || p->wind != 0.0) && !p->d_aux) return TF_ERR_ARG;
    const bool cor = p->rossby != 0.0;
#define TF_CALL(D, F) launch_assemble<D, F>(cor, blocks, s, *p, d_state, d_rhs, d_jvals); launched()
    TF_DISPATCH(p->dim, p->dof, TF_CALL);
#undef TF_CALL
    return cuda_status();
}

extern "C" int tf_mass_diag(const tf_problem *p, double *d_diag, tf_stream_t stream) {
    int e = check_problem(p);
    if (e) return e;
    if (!d_diag) return TF_ERR_ARG;
    const int ncell = p->nx * p->ny * p->nz;
    const int blocks = (ncell + 127) / 128;
#define TF_CALL(D, F) mass_kernel<D, F><<<blocks, 128, 0, (cudaStream_t)stream>>>(*p, d_diag); launched()
    TF_DISPATCH(p->dim, p->dof, TF_CALL);
#undef TF_CALL
    return cuda_status();
}
