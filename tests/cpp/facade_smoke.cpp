// Drop-in check of the C++ facade: the reference's call sequence
// (examples/roots_newton_circle.cpp:92-138) written against include/hbem.hpp.
#include <cmath>
#include <cstdio>

#include "hbem.hpp"

int main(int argc, char** argv) {
    using namespace hbem;
    Mesh mesh = Mesh::circle(0., 0., 0.25, 16);
    BuilderData builder_data(mesh, P1, P1, 7);
    SolutionsOperator so(builder_data);
    MatrixXcd T, T_der, T_der2;
    so.gen_sol_op_2nd_der(2.5, 1.0, 23.4, T, T_der, T_der2);
    auto r = direct::sv_2nd_der(T, T_der, T_der2);
    GalerkinBuilder builder(builder_data);
    builder.assembleDense(2.5, 23.4, LayerType::ALL, 1);
    const MatrixXcd& V1 = builder.getSingleLayer(1);
    bool found = false;
    unsigned it = 0;
    double root = rtsafe([](double x) { return std::cos(x); },
                         [](double x) { return std::vector<double>{std::cos(x), -std::sin(x)}; }, 1.0, 2.0, 1e-12,
                         found, it);
    bool threw = false;
    try {
        builder.assembleDense(1.0, 0.5);   // c < 1: the reference throws std::runtime_error
    } catch (const std::runtime_error&) {
        threw = true;
    }
    // arnoldi::sv as in examples/roots_brent_circle_arnoldi.cpp:121 (count 1)
    const double a0 = arnoldi::sv(T, 1, 1e-12)[0];
    const MatrixXd a2 = arnoldi::sv_2nd_der(T, T_der, T_der2, 1, 1e-12);
    // scatterer file -> corner-graded polygon mesh, as examples/roots_brent_polygon.cpp:72-121 does
    double sq_sigma = -1.;
    int sq_panels = -1;
    if (argc > 1) {
        if (FILE* fp = std::fopen(argv[1], "w")) {
            std::fputs("0,0\n 1, 0\n\n1,1\r\n0,1\n", fp);
            std::fclose(fp);
        }
        VectorXd px, py;
        if (scatterer::read(argv[1], px, py, 0.5)) {
            Mesh sq = scatterer::make_polygonal_panels(px, py, 24, 0.5);
            sq_panels = sq.size();
            BuilderData sq_data(sq, P1, P1, 7);
            SolutionsOperator sq_so(sq_data);
            MatrixXcd Tsq;
            sq_so.gen_sol_op(3.0, 1.0, 4.0, Tsq);
            sq_sigma = direct::sv(Tsq);
        }
    }
    // transmission problem on the circle and its total field (examples/plot_solution_polygon.cpp:169-181)
    incoming::wave w(1);
    w[0].type = incoming::WaveType::Plane;
    w[0].angle = 0.5;
    const double ll[2] = {-0.5, -0.5}, ur[2] = {0.5, 0.5};
    MatrixXd gX, gY;
    MatrixXcd S = tp::direct_second_kind::solve_in_rectangle(mesh, w, 7, 10, 2.5, 1.0, 4.0, ll, ur, 9, 7, gX, gY, true);
    // randomized_svd::sv on a seeded sketch, and BrentMinimizer's reverse communication as in
    // examples/find_resonances.cpp:116-121
    MatrixXcd R = randomized_svd::randGaussian((int)T.rows(), 12, 3);
    const double rs = randomized_svd::sv(T, R, 2);
    BrentMinimizer br(2.0, 4.0, 1e-8);
    int status = 0;
    double arg = br.local_min_rc(status, 0.);
    while (status) arg = br.local_min_rc(status, std::cos(arg));
    std::printf("%.17e %.17e %.17e %.17e %.17e %d %d %.17e %.17e %d %.17e %.17e %.17e %.17e %.17e %.17e\n", r[0], r[1],
                r[2], std::abs(V1(3, 5)), root, (int)found, (int)threw, a0, a2(0, 0), sq_panels, sq_sigma,
                S(2, 5).real(), S(2, 5).imag(), gY(2, 5), rs, arg);
    return (found && threw) ? 0 : 1;
}
