// Compile check of include/nsl_gb300/nsl_dropin.hpp against the reference NSL headers: the drop-in classes must
// instantiate inside the reference's own HubbardFermionAction, Action sum and Leapfrog templates. Test
// infrastructure (built with -fsyntax-only by tests/test_dropin_cpp.py).
#include "nsl_shims.hpp"

#include "Tensor.hpp"
#include "LinAlg.hpp"
#include "Lattice.hpp"
#include "FermionMatrix.hpp"
#include "Configuration.hpp"
#include "Action.hpp"
#include "Integrator.hpp"

#include "nsl_gb300/nsl_dropin.hpp"

using C = NSL::complex<double>;
using Lat = NSL::Lattice::Honeycomb<C>;
using HFM = NSL::FermionMatrix::HubbardExpGB300<C, Lat>;

int main() {
    Lat lat({3, 3});
    NSL::Parameter params;
    params["beta"] = C(4.0);
    params["U"] = C(2.0);
    params["mu"] = C(0.0);
    params["Nt"] = NSL::size_t(16);

    HFM hfm(lat, params);
    NSL::Tensor<C> phi(16, 18), psi(4, 16, 18);
    hfm.populate(phi, NSL::Hubbard::Particle);
    NSL::Tensor<C> y = hfm.MMdagger(psi);
    C ld = hfm.logDetM();
    NSL::Tensor<C> g = hfm.gradLogDetM();

    NSL::LinAlg::CGGB300<C> cg(hfm, NSL::FermionMatrix::MMdagger, 1e-12, 10000);
    NSL::Tensor<C> x = cg(psi);

    NSL::Action::HubbardGaugeAction<C> S_gauge(params);
    NSL::Action::HubbardFermionAction<C, Lat, HFM> S_fermion(lat, params);
    NSL::Action::Action S = S_gauge + S_fermion;
    NSL::Configuration<C> q{{"phi", phi}}, p{{"phi", phi}};
    NSL::Integrator::Leapfrog lf(S, 1.0, 10);
    auto [q1, p1] = lf(q, p);
    (void)ld;

    // the diagonal discretisation in the same template slots
    using HFD = NSL::FermionMatrix::HubbardDiagGB300<C, Lat>;
    HFD hfd(lat, params);
    hfd.populate(phi, NSL::Hubbard::Hole);
    NSL::Tensor<C> yd = hfd.MdaggerM(psi);
    NSL::LinAlg::CGGB300<C> cgd(hfd, NSL::FermionMatrix::MMdagger, 1e-12, 10000);
    NSL::Tensor<C> xd = cgd(psi);
    NSL::Action::HubbardFermionAction<C, Lat, HFD> S_fermion_d(lat, params);
    NSL::Action::Action Sd = S_gauge + S_fermion_d;
    NSL::Integrator::LeapfrogRealForce lfd(Sd, 1.0, 10);
    auto [q2, p2] = lfd(q, p);

    // two-body correlators from momentum wall sources
    params["wallSources"] = NSL::Tensor<C>(4, 2, 18);
    params["momenta"] = NSL::Tensor<double>(4, 2);
    NSL::Measure::Hubbard::TwoBodyCorrelatorGB300<C, Lat> tb(lat, params);
    tb.measure(phi, 4);
    const auto &ch = tb.channel(NSLG_TB_I1S1IZ1SZ1);
    (void)ch;

    // two-point correlators: point sources and momentum wall sources
    NSL::Measure::Hubbard::TwoPointCorrelatorGB300<C, Lat> tp(lat, params, NSL::Hubbard::Hole);
    tp.measure(phi, 4);
    tp.measureK(phi, 1, 4);
    NSL::Tensor<C> corr = tp.corr(), block = tp.corrKblock();
    return 0;
}
