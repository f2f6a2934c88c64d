// Golden-vector harness: TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference NSL headers, unmodified and read in place from the reference checkout, against the
// in-image libtorch (CPU) and evaluates the reference's own fermion-matrix hot path on inputs written by
// tests/golden/make_golden.py. Its outputs are committed as small fixtures under tests/golden/ and pin the
// oracle restatement (oracle/nsl_oracle.py). Nothing in the product links or runs this program.
//
// Dependencies absent from this image are shimmed by nsl_shims.hpp (no reference file is edited); its logger
// records the last message, so the CG iteration count logged at src/NSL/LinAlg/Solver/Impl/CG.tpp:71 can be read.
//
// Usage: golden_harness <case-dir>. The directory holds params.txt (key value lines) and raw little-endian
// complex128 inputs (phi.bin, psi.bin, b.bin, p.bin); the harness writes raw complex128 outputs next to them.

#include "nsl_shims.hpp"

#include <array>
#include <chrono>
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "Tensor.hpp"
#include "LinAlg.hpp"
#include "Lattice.hpp"
#include "FermionMatrix.hpp"
#include "Configuration.hpp"
#include "Action.hpp"
#include "Integrator.hpp"

// The two-body correlator's base class holds an NSL::H5IO reference (src/NSL/Measurements/measure.hpp), whose
// HighFive backend is absent here. measure(NumberTimeSources) never touches it; this stand-in only lets the
// class compile (its members are the calls the file-level measure() would make).
namespace NSL {
class H5IO {
  public:
    bool exist(const std::string &) { return false; }
    template <class T> void write(const T &, const std::string &) {}
    template <class T> void read(T &, const std::string &) {}
    std::pair<NSL::size_t, NSL::size_t> getMinMaxConfigs(const std::string &) { return {0, 0}; }
    void deleteData(const std::string &) {}
};
}  // namespace NSL
#include "Measurements/Hubbard/twoBodyCorrelationFunction.tpp"
#include "Measurements/Hubbard/twoPointCorrelationFunction.tpp"

using C = NSL::complex<double>;

namespace {

std::map<std::string, std::vector<std::string>> read_params(const std::string &dir) {
    std::map<std::string, std::vector<std::string>> p;
    std::ifstream in(dir + "/params.txt");
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ss(line);
        std::string key, tok;
        if (!(ss >> key)) continue;
        std::vector<std::string> vals;
        while (ss >> tok) vals.push_back(tok);
        p[key] = vals;
    }
    return p;
}

torch::Tensor read_c128(const std::string &path, std::vector<int64_t> shape) {
    int64_t n = 1;
    for (auto s : shape) n *= s;
    std::vector<double> buf(2 * n);
    std::FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::runtime_error("cannot open " + path);
    size_t got = std::fread(buf.data(), sizeof(double), buf.size(), f);
    std::fclose(f);
    if (got != buf.size()) throw std::runtime_error("short read " + path);
    auto t = torch::from_blob(buf.data(), {n, 2}, torch::kDouble).clone();
    return torch::view_as_complex(t).reshape(shape).contiguous();
}

void write_c128(const std::string &path, const torch::Tensor &t) {
    auto c = t.to(torch::kComplexDouble).contiguous();
    auto r = torch::view_as_real(c).contiguous();
    std::FILE *f = std::fopen(path.c_str(), "wb");
    std::fwrite(r.data_ptr<double>(), sizeof(double), r.numel(), f);
    std::fclose(f);
}

void write_scalar(const std::string &path, C v) {
    write_c128(path, torch::tensor({c10::complex<double>(v.real(), v.imag())}, torch::kComplexDouble));
}

long parse_cg_steps(const std::string &msg) {
    auto pos = msg.rfind("after ");
    if (pos == std::string::npos) return -1;
    return std::stol(msg.substr(pos + 6));
}

template <class Lattice>
void run(const std::string &dir, std::map<std::string, std::vector<std::string>> &P, Lattice &lat) {
    const int64_t Nt = std::stol(P["Nt"][0]);
    const double beta = std::stod(P["beta"][0]);
    const double mu = std::stod(P["mu"][0]);
    const double U = std::stod(P["U"][0]);
    const int64_t R = std::stol(P["nrhs"][0]);
    const int64_t Nx = lat.sites();

    NSL::Parameter params;
    params["beta"] = C(beta);
    params["U"] = C(U);
    params["mu"] = C(mu);
    params["Nt"] = Nt;

    const C delta = C(beta) / C(double(Nt));
    write_c128(dir + "/hops.bin", torch::Tensor(lat.hopping_matrix(C(1.0))));
    write_c128(dir + "/expK_pos.bin", torch::Tensor(lat.exp_hopping_matrix(delta)));
    write_c128(dir + "/expK_neg.bin", torch::Tensor(lat.exp_hopping_matrix(C(-1.0) * delta)));

    NSL::Tensor<C> phi(read_c128(dir + "/phi.bin", {Nt, Nx}));
    NSL::Tensor<C> psi(read_c128(dir + "/psi.bin", {R, Nt, Nx}));

    // Fermion matrix applications and log-determinant for both species (hubbardExp.tpp:13-211).
    NSL::FermionMatrix::HubbardExp<C, Lattice> hfm(lat, Nt, C(beta), C(mu));
    const char *tag[2] = {"P", "H"};
    NSL::Hubbard::Species sp[2] = {NSL::Hubbard::Particle, NSL::Hubbard::Hole};
    for (int s = 0; s < 2; ++s) {
        hfm.populate(phi, sp[s]);
        write_c128(dir + "/M_" + std::string(tag[s]) + ".bin", torch::Tensor(hfm.M(psi)));
        write_c128(dir + "/Mdag_" + std::string(tag[s]) + ".bin", torch::Tensor(hfm.Mdagger(psi)));
        write_c128(dir + "/MMdag_" + std::string(tag[s]) + ".bin", torch::Tensor(hfm.MMdagger(psi)));
        write_c128(dir + "/MdagM_" + std::string(tag[s]) + ".bin", torch::Tensor(hfm.MdaggerM(psi)));
        if (P.count("logdet")) {
            write_scalar(dir + "/logdet_" + std::string(tag[s]) + ".bin", hfm.logDetM());
            write_c128(dir + "/grad_" + std::string(tag[s]) + ".bin", torch::Tensor(hfm.gradLogDetM()));
        }
    }

    // The diagonal discretisation for both species (hubbardDiag.tpp:10-254). Its operators shift along dimension 0
    // and index slice 0 of dimension 0 (written for a single (Nt, Nx) vector), so they are evaluated one
    // right-hand side at a time and stacked.
    NSL::FermionMatrix::HubbardDiag<C, Lattice> hfd(lat, Nt, C(beta), C(mu));
    auto per_rhs = [&](auto op) {
        std::vector<torch::Tensor> outs;
        for (int64_t r = 0; r < R; ++r) {
            NSL::Tensor<C> v(torch::Tensor(psi).select(0, r).contiguous().clone());
            outs.push_back(torch::Tensor(op(v)).clone());
        }
        return torch::stack(outs);
    };
    for (int s = 0; s < 2; ++s) {
        hfd.populate(phi, sp[s]);
        write_c128(dir + "/diag_M_" + std::string(tag[s]) + ".bin", per_rhs([&](NSL::Tensor<C> &v) { return hfd.M(v); }));
        write_c128(dir + "/diag_Mdag_" + std::string(tag[s]) + ".bin",
                   per_rhs([&](NSL::Tensor<C> &v) { return hfd.Mdagger(v); }));
        write_c128(dir + "/diag_MMdag_" + std::string(tag[s]) + ".bin",
                   per_rhs([&](NSL::Tensor<C> &v) { return hfd.MMdagger(v); }));
        write_c128(dir + "/diag_MdagM_" + std::string(tag[s]) + ".bin",
                   per_rhs([&](NSL::Tensor<C> &v) { return hfd.MdaggerM(v); }));
        if (P.count("logdet")) {
            write_scalar(dir + "/diag_logdet_" + std::string(tag[s]) + ".bin", hfd.logDetM());
            write_c128(dir + "/diag_grad_" + std::string(tag[s]) + ".bin", torch::Tensor(hfd.gradLogDetM()));
        }
    }

    // CG on MM^dagger, particle species, with the reference's own stopping rule (CG.tpp:15-95).
    if (P.count("cg_eps")) {
        const double eps = std::stod(P["cg_eps"][0]);
        const int64_t maxIter = std::stol(P["cg_maxiter"][0]);
        NSL::Tensor<C> b(read_c128(dir + "/b.bin", {R, Nt, Nx}));
        hfm.populate(phi, NSL::Hubbard::Particle);
        NSL::LinAlg::CG<C> cg(hfm, NSL::FermionMatrix::MMdagger, eps, maxIter);
        const auto t0 = std::chrono::steady_clock::now();
        NSL::Tensor<C> x = cg(b);
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        write_c128(dir + "/cg_x.bin", torch::Tensor(x).clone());
        std::ofstream(dir + "/cg_iters.txt") << parse_cg_steps(NSL::Logger::last_message) << "\n"
                                             << NSL::Logger::last_message << "\n";
        std::ofstream(dir + "/cg_seconds.txt") << secs << "\n";  // wall time of the solve (one thread)
    }

    // Action value, force and leapfrog trajectories (hubbardFermiAction.tpp, hubbardGaugeAction.tpp, leapfrog.tpp).
    if (P.count("nmd")) {
        const int64_t Nmd = std::stol(P["nmd"][0]);
        const double tau = std::stod(P["traj"][0]);
        NSL::Action::HubbardGaugeAction<C> S_gauge(params);
        NSL::Action::HubbardFermionAction<C, Lattice, NSL::FermionMatrix::HubbardExp<C, Lattice>> S_fermion(lat, params);
        NSL::Action::Action S = S_gauge + S_fermion;

        NSL::Configuration<C> q{{"phi", phi}};
        NSL::Configuration<C> p{{"phi", NSL::Tensor<C>(read_c128(dir + "/p.bin", {Nt, Nx}))}};

        write_scalar(dir + "/S.bin", S(q));
        write_scalar(dir + "/S_gauge.bin", S_gauge.eval(q));
        write_scalar(dir + "/S_fermion.bin", S_fermion.eval(q));
        write_c128(dir + "/force.bin", torch::Tensor(S.force(q)["phi"]));
        write_c128(dir + "/force_fermion.bin", torch::Tensor(S_fermion.force(q)["phi"]));

        NSL::Integrator::Leapfrog lf(S, tau, Nmd);
        auto [q1, p1] = lf(q, p);
        write_c128(dir + "/lf_q.bin", torch::Tensor(q1["phi"]));
        write_c128(dir + "/lf_p.bin", torch::Tensor(p1["phi"]));
        write_scalar(dir + "/lf_S.bin", S(q1));

        NSL::Integrator::LeapfrogRealForce lfr(S, tau, Nmd);
        auto [q2, p2] = lfr(q, p);
        write_c128(dir + "/lfr_q.bin", torch::Tensor(q2["phi"]));
        write_c128(dir + "/lfr_p.bin", torch::Tensor(p2["phi"]));
        write_scalar(dir + "/lfr_S.bin", S(q2));
    }
}

// TwoBodyCorrelator::measure(NumberTimeSources) on phi (twoBodyCorrelationFunction.tpp:188-306) with the fermion
// matrix FM (HubbardExp, or HubbardDiag with "twobody nk nb nts diag"); a derived class reads the protected
// configuration and correlator maps.
template <class Lattice, class FM>
struct TwoBodyProbe : NSL::Measure::Hubbard::TwoBodyCorrelator<C, Lattice, FM> {
    using Base = NSL::Measure::Hubbard::TwoBodyCorrelator<C, Lattice, FM>;
    using Base::Base;
    void set_phi(const NSL::Tensor<C> &phi) { this->phi_ = phi; }
    // channel maps in the order measure(NumberTimeSources) evaluates them (:290-303)
    auto channels() {
        using Map = std::remove_reference_t<decltype(this->cI1S1Iz1Sz1_)>;
        return std::vector<Map *>{&this->cI1S1Iz1Sz1_, &this->cI1S1Iz1Sz0_, &this->cI1S1Iz1Szn1_, &this->cI1S1Iz0Sz1_,
                &this->cI1S1Iz0Szn1_, &this->cI1S1Izn1Sz1_, &this->cI1S1Izn1Sz0_, &this->cI1S1Izn1Szn1_,
                &this->cI0S1Iz0Sz1_, &this->cI0S1Iz0Szn1_, &this->cI1S0Iz1Sz0_, &this->cI1S0Izn1Sz0_};
    }
};

template <class Lattice, class FM>
void run_twobody(const std::string &dir, std::map<std::string, std::vector<std::string>> &P, Lattice &lat) {
    const int64_t Nt = std::stol(P["Nt"][0]);
    const int64_t Nx = lat.sites();
    const int64_t nk = std::stol(P["twobody"][0]), nb = std::stol(P["twobody"][1]), nts = std::stol(P["twobody"][2]);
    NSL::Parameter params;
    params["beta"] = C(std::stod(P["beta"][0]));
    params["mu"] = C(std::stod(P["mu"][0]));
    params["Nt"] = Nt;
    params["Nx"] = Nx;
    params["device"] = NSL::CPU();
    params["wallSources"] = NSL::Tensor<C>(read_c128(dir + "/wall.bin", {nk, nb, Nx}));
    std::vector<double> mom(2 * nk);
    std::FILE *f = std::fopen((dir + "/momenta.bin").c_str(), "rb");
    if (!f || std::fread(mom.data(), sizeof(double), mom.size(), f) != mom.size()) throw std::runtime_error("momenta");
    std::fclose(f);
    NSL::Tensor<double> momenta(nk, 2);
    for (int64_t k = 0; k < nk; ++k) {
        momenta(k, 0) = mom[2 * k];
        momenta(k, 1) = mom[2 * k + 1];
    }
    params["momenta"] = momenta;
    NSL::H5IO h5;
    TwoBodyProbe<Lattice, FM> corr(lat, params, h5, std::string("twobody"));
    corr.set_phi(NSL::Tensor<C>(read_c128(dir + "/phi.bin", {Nt, Nx})));
    corr.measure(nts);
    // every allocated key in lexicographic order, then the twelve channels' tensors for those keys
    auto chans = corr.channels();
    auto &first = *chans[0];
    std::vector<std::array<int, 4>> keys;
    for (int w = 0; w < nk; ++w)
        for (int x = 0; x < nk; ++x)
            for (int p = 0; p < nk; ++p)
                for (int q = 0; q < nk; ++q)
                    if (first.count(w) && first[w].count(x) && first[w][x].count(p) && first[w][x][p].count(q))
                        keys.push_back({w, x, p, q});
    std::ofstream kt(dir + "/tb_tuples.txt");
    for (auto &k : keys) kt << k[0] << " " << k[1] << " " << k[2] << " " << k[3] << "\n";
    std::vector<torch::Tensor> all;
    for (auto *m : chans)
        for (auto &k : keys) all.push_back(torch::Tensor((*m)[k[0]][k[1]][k[2]][k[3]]).clone());
    write_c128(dir + "/tb_out.bin", torch::stack(all));
}

// TwoPointCorrelator::measure(NumberTimeSources) (point sources, twoPointCorrelationFunction.tpp:116-162) and
// measureK(k, NumberTimeSources) (momentum wall sources, :169-233) on phi for one species; a derived class sets the
// protected configuration and reads the correlators.
template <class Lattice, class FM>
struct TwoPointProbe : NSL::Measure::Hubbard::TwoPointCorrelator<C, Lattice, FM> {
    using Base = NSL::Measure::Hubbard::TwoPointCorrelator<C, Lattice, FM>;
    using Base::Base;
    void set_phi(const NSL::Tensor<C> &phi) { this->phi_ = phi; }
    torch::Tensor corr() { return torch::Tensor(this->corr_).clone(); }
    torch::Tensor block() { return torch::Tensor(this->corrKblock_).clone(); }
};

// "twopoint nk nb nts": both species' point-source correlators (tp_corr_P.bin, tp_corr_H.bin: Nt x Nx x Nx) and
// their momentum blocks for every wall source k (tpk_P.bin, tpk_H.bin: nk x Nt x nb x nb).
template <class Lattice, class FM>
void run_twopoint(const std::string &dir, std::map<std::string, std::vector<std::string>> &P, Lattice &lat) {
    const int64_t Nt = std::stol(P["Nt"][0]);
    const int64_t Nx = lat.sites();
    const int64_t nk = std::stol(P["twopoint"][0]), nb = std::stol(P["twopoint"][1]);
    const int64_t nts = std::stol(P["twopoint"][2]);
    NSL::Parameter params;
    params["beta"] = C(std::stod(P["beta"][0]));
    params["mu"] = C(std::stod(P["mu"][0]));
    params["Nt"] = Nt;
    params["Nx"] = Nx;
    params["device"] = NSL::CPU();
    params["wallSources"] = NSL::Tensor<C>(read_c128(dir + "/wall.bin", {nk, nb, Nx}));
    const NSL::Tensor<C> phi(read_c128(dir + "/phi.bin", {Nt, Nx}));
    const std::pair<NSL::Hubbard::Species, const char *> species[] = {{NSL::Hubbard::Particle, "P"},
                                                                      {NSL::Hubbard::Hole, "H"}};
    for (auto [sp, tag] : species) {
        NSL::H5IO h5;
        TwoPointProbe<Lattice, FM> corr(lat, params, h5, sp, std::string("twopoint"));
        corr.set_phi(phi);
        corr.measure(nts);
        write_c128(dir + "/tp_corr_" + tag + ".bin", corr.corr());
        // A second correlator for the wall sources: the CG member deep-copies each right-hand side into the
        // solution buffer of its first solve (CG.tpp:102, tensor.hpp:115-123), so one object cannot follow Nx point
        // sources with nb wall sources (the reference's example_k_correlators.cpp calls only measureK()).
        TwoPointProbe<Lattice, FM> corrk(lat, params, h5, sp, std::string("twopoint"));
        corrk.set_phi(phi);
        std::vector<torch::Tensor> blocks;
        for (int64_t k = 0; k < nk; ++k) {
            corrk.measureK(k, nts);
            blocks.push_back(corrk.block());
        }
        write_c128(dir + "/tpk_" + tag + ".bin", torch::stack(blocks));
    }
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: %s <case-dir>\n", argv[0]);
        return 2;
    }
    torch::set_num_threads(1);
    const std::string dir = argv[1];
    auto P = read_params(dir);
    const auto &L = P.at("lattice");
    if (L[0] == "ring") {
        NSL::Lattice::Ring<C> lat(std::stol(L[1]));
        run(dir, P, lat);
    } else if (L[0] == "honeycomb") {
        NSL::Lattice::Honeycomb<C> lat(std::vector<int>{std::stoi(L[1]), std::stoi(L[2])});
        using L = NSL::Lattice::Honeycomb<C>;
        if (P.count("twobody") && P["twobody"].size() > 3 && P["twobody"][3] == "diag")
            run_twobody<L, NSL::FermionMatrix::HubbardDiag<C, L>>(dir, P, lat);
        else if (P.count("twobody"))
            run_twobody<L, NSL::FermionMatrix::HubbardExp<C, L>>(dir, P, lat);
        else if (P.count("twopoint"))
            run_twopoint<L, NSL::FermionMatrix::HubbardExp<C, L>>(dir, P, lat);
        else run(dir, P, lat);
    } else {
        std::fprintf(stderr, "unknown lattice %s\n", L[0].c_str());
        return 2;
    }
    return 0;
}
