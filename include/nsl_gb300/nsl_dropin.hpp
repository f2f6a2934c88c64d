// NSL-side binding of libnslgpu: drop-in replacements for the reference's fermion-matrix hot path, over NSL::Tensor.
//
// Include this header after the NSL headers. It provides
//   NSL::FermionMatrix::HubbardExpGB300<Type, LatticeType>   (replaces HubbardExp, hubbardExp.{hpp,tpp})
//   NSL::LinAlg::CGGB300<Type>                                (replaces CG for HubbardExpGB300, CG.{hpp,tpp})
//   NSL::Measure::Hubbard::TwoBodyCorrelatorGB300<...>        (TwoBodyCorrelator::measure(NumberTimeSources),
//                                                             twoBodyCorrelationFunction.tpp, without HDF5)
//   NSL::Measure::Hubbard::TwoPointCorrelatorGB300<...>       (TwoPointCorrelator::measure(NumberTimeSources) and
//                                                             measureK(k, NumberTimeSources),
//                                                             twoPointCorrelationFunction.tpp, without HDF5)
// with the reference's constructors and member signatures, so HubbardFermionAction<Type, Lattice, HubbardExpGB300<...>>,
// Leapfrog and HMC instantiate unchanged. Tensors are passed by their data() pointers (host or device storage);
// results come back as NSL::Tensor on the input's device. Link with -lnslgpu.
#pragma once

#include <cmath>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "../nsl_gb300.h"

namespace NSL::GB300 {

inline void check(int rc) {
    if (rc != NSLG_OK && rc != NSLG_NOT_CONVERGED) throw std::runtime_error(std::string("libnslgpu: ") + nslg_last_error());
}

inline nslg_c128 c128(const NSL::complex<double> &z) { return nslg_c128{z.real(), z.imag()}; }

// One context per process and device; its stream orders every call.
inline nslg_ctx *context(int device = 0) {
    static nslg_ctx *ctx = nullptr;
    if (!ctx) check(nslg_ctx_create(device, nullptr, &ctx));
    return ctx;
}

inline nslg_c128 *ptr(const NSL::Tensor<NSL::complex<double>> &t) {
    return reinterpret_cast<nslg_c128 *>(const_cast<NSL::complex<double> *>(t.data()));
}

}  // namespace NSL::GB300

namespace NSL::FermionMatrix {

template <NSL::Concept::isNumber Type, NSL::Concept::isDerived<NSL::Lattice::SpatialLattice<Type>> LatticeType>
class HubbardExpGB300 : public FermionMatrix<Type, LatticeType> {
    static_assert(std::is_same_v<Type, NSL::complex<double>>, "libnslgpu computes in complex128");

  public:
    HubbardExpGB300() = delete;

    // hubbardExp.hpp:48-84
    HubbardExpGB300(LatticeType &lat, const NSL::size_t Nt, const Type &beta = 1.0, const Type &mu = 0.0)
        : HubbardExpGB300(NSL::Hubbard::Species::Particle, lat, Nt, beta, mu) {}
    HubbardExpGB300(NSL::Hubbard::Species species, LatticeType &lat, const NSL::size_t Nt, const Type &beta = 1.0,
                    const Type &mu = 0.0)
        : HubbardExpGB300(NSLG_FM_EXP, species, lat, Nt, beta, mu) {}
    HubbardExpGB300(NSL::Hubbard::Species species, LatticeType &lat, NSL::Parameter &params)
        : HubbardExpGB300(species, lat, params["Nt"], params["beta"], params["mu"]) {}
    HubbardExpGB300(LatticeType &lat, NSL::Parameter &params)
        : HubbardExpGB300(lat, params["Nt"], params["beta"], params["mu"]) {}
    HubbardExpGB300(const HubbardExpGB300 &o) : HubbardExpGB300(o.kind_, o.species_, o.Lat, o.Nt_, o.beta_(), o.mu_()) {
        if (o.populated_) populate(o.phi_);
    }
    ~HubbardExpGB300() { nslg_fm_destroy(fm_); }

    // hubbardExp.hpp:95-144
    void populate(const NSL::Tensor<Type> &phi, const NSL::Hubbard::Species &species) {
        species_ = species;
        phi_ = phi;
        NSL::GB300::check(nslg_fm_populate(fm_, NSL::GB300::ptr(phi_),
                                           species == NSL::Hubbard::Particle ? NSLG_PARTICLE : NSLG_HOLE));
        populated_ = true;
    }
    void populate(const NSL::Tensor<Type> &phi) { populate(phi, species_); }
    void populate(const NSL::Tensor<Type> &phi, const NSL::Hubbard::Species &species, bool) { populate(phi, species); }
    void populate(const NSL::Tensor<Type> &phi, bool) { populate(phi); }

    // hubbardExp.tpp:39-125
    NSL::Tensor<Type> M(const NSL::Tensor<Type> &psi) override { return apply_(NSLG_OP_M, psi); }
    NSL::Tensor<Type> Mdagger(const NSL::Tensor<Type> &psi) override { return apply_(NSLG_OP_MDAGGER, psi); }
    NSL::Tensor<Type> MMdagger(const NSL::Tensor<Type> &psi) override { return apply_(NSLG_OP_MMDAGGER, psi); }
    NSL::Tensor<Type> MdaggerM(const NSL::Tensor<Type> &psi) override { return apply_(NSLG_OP_MDAGGERM, psi); }

    // hubbardExp.tpp:129-211
    Type logDetM() override {
        nslg_c128 out;
        NSL::GB300::check(nslg_fm_logdet(fm_, &out));
        return Type(out.re, out.im);
    }
    NSL::Tensor<Type> gradLogDetM() override {
        NSL::Tensor<Type> out(phi_.device(), Nt_, Nx_);
        NSL::GB300::check(nslg_fm_grad_logdet(fm_, NSL::GB300::ptr(out)));
        return out;
    }

    NSL::Hubbard::Species species() { return species_; }
    nslg_fm *handle() { return fm_; }

  protected:
    // nslg_fm_create_kind: the exponential (NSLG_FM_EXP) or the diagonal (NSLG_FM_DIAG) discretisation
    HubbardExpGB300(int kind, NSL::Hubbard::Species species, LatticeType &lat, const NSL::size_t Nt, const Type &beta,
                    const Type &mu)
        : FermionMatrix<Type, LatticeType>(lat), kind_(kind), species_(species), Nt_(Nt), Nx_(lat.sites()),
          phi_(lat.device(), Nt, lat.sites()), beta_store_(beta), mu_store_(mu) {
        NSL::Tensor<Type> K = lat.hopping_matrix(Type(1.0));
        NSL::GB300::check(nslg_fm_create_kind(NSL::GB300::context(), kind, Nx_, Nt_, NSL::GB300::ptr(K),
                                              NSL::GB300::c128(beta), NSL::GB300::c128(mu),
                                              species == NSL::Hubbard::Particle ? NSLG_PARTICLE : NSLG_HOLE, &fm_));
        if (kind != NSLG_FM_EXP) return;
        // Reuse the lattice's memoised exp(delta K) so both implementations see the same matrix.
        const Type delta = beta / Type(double(Nt));
        for (const Type d : {delta, Type(-1.0) * delta}) {
            NSL::Tensor<Type> E = lat.exp_hopping_matrix(d);
            NSL::GB300::check(nslg_fm_set_exp_hopping(fm_, NSL::GB300::c128(d), NSL::GB300::ptr(E)));
        }
    }

  private:
    NSL::Tensor<Type> apply_(int op, const NSL::Tensor<Type> &psi) {
        NSL::Tensor<Type> in(psi, true);  // contiguous deep copy: the ABI reads plain row-major storage
        NSL::Tensor<Type> out(in, true);
        const int64_t nbatch = in.numel() / (Nt_ * Nx_);
        NSL::GB300::check(nslg_fm_apply(fm_, op, NSL::GB300::ptr(in), NSL::GB300::ptr(out), nbatch, NSLG_PREC_FP64));
        return out;
    }
    Type beta_() const { return beta_store_; }
    Type mu_() const { return mu_store_; }

    int kind_ = NSLG_FM_EXP;
    NSL::Hubbard::Species species_;
    NSL::size_t Nt_, Nx_;
    NSL::Tensor<Type> phi_;
    bool populated_ = false;
    Type beta_store_ = 1.0, mu_store_ = 0.0;
    nslg_fm *fm_ = nullptr;
};

// NSL::FermionMatrix::HubbardDiag (hubbardDiag.hpp:44-93, hubbardDiag.tpp): the diagonal discretisation on the same
// C ABI (nslg_fm_create_kind with NSLG_FM_DIAG); constructors, populate, operators, logDetM and gradLogDetM as above.
// The reference's operators take one (Nt, Nx) vector; a leading batch dimension here holds independent vectors.
template <NSL::Concept::isNumber Type, NSL::Concept::isDerived<NSL::Lattice::SpatialLattice<Type>> LatticeType>
class HubbardDiagGB300 : public HubbardExpGB300<Type, LatticeType> {
    using Base = HubbardExpGB300<Type, LatticeType>;

  public:
    HubbardDiagGB300() = delete;
    HubbardDiagGB300(LatticeType &lat, const NSL::size_t Nt, const Type &beta = 1.0, const Type &mu = 0.0)
        : Base(NSLG_FM_DIAG, NSL::Hubbard::Species::Particle, lat, Nt, beta, mu) {}
    HubbardDiagGB300(NSL::Hubbard::Species species, LatticeType &lat, const NSL::size_t Nt, const Type &beta = 1.0,
                     const Type &mu = 0.0)
        : Base(NSLG_FM_DIAG, species, lat, Nt, beta, mu) {}
    HubbardDiagGB300(NSL::Hubbard::Species species, LatticeType &lat, NSL::Parameter &params)
        : HubbardDiagGB300(species, lat, params["Nt"], params["beta"], params["mu"]) {}
    HubbardDiagGB300(LatticeType &lat, NSL::Parameter &params)
        : HubbardDiagGB300(lat, params["Nt"], params["beta"], params["mu"]) {}
};

}  // namespace NSL::FermionMatrix

namespace NSL::LinAlg {

// CG(M, MatrixCombination, eps, maxIter) for HubbardExpGB300 (CG.hpp:142-186): the reference's semantics (shared
// alpha/beta over the batch, recurrence rule, x0 = b, log-and-return on exhaustion).
template <NSL::Concept::isNumber Type> class CGGB300 {
  public:
    template <typename FM>
    CGGB300(FM &M, NSL::FermionMatrix::MatrixCombination comb = NSL::FermionMatrix::M,
            const NSL::RealTypeOf<Type> eps = 1e-12, const NSL::size_t maxIter = 10000)
        : fm_(M.handle()), op_(static_cast<int>(comb)), eps_(eps), maxIter_(maxIter) {}

    NSL::Tensor<Type> operator()(const NSL::Tensor<Type> &b) { return solve_(b, nullptr); }
    NSL::Tensor<Type> operator()(const NSL::Tensor<Type> &b, const NSL::Tensor<Type> &x0) { return solve_(b, &x0); }

    nslg_cg_stats stats{};

  private:
    NSL::Tensor<Type> solve_(const NSL::Tensor<Type> &b, const NSL::Tensor<Type> *x0) {
        NSL::Tensor<Type> bb(b, true), x(b, true);
        NSL::Tensor<Type> x0c;
        if (x0) x0c = NSL::Tensor<Type>(*x0, true);
        const int64_t nbatch = bb.numel() / (bb.shape(-1) * bb.shape(-2));
        NSL::GB300::check(nslg_cg_solve(fm_, op_, NSL::GB300::ptr(bb), x0 ? NSL::GB300::ptr(x0c) : nullptr,
                                        NSL::GB300::ptr(x), nbatch, eps_, maxIter_, NSLG_CG_SHARED, NSLG_PREC_FP64,
                                        NSLG_STOP_RECURRENCE, &stats));
        return x;
    }
    nslg_fm *fm_;
    int op_;
    double eps_;
    int64_t maxIter_;
};

}  // namespace NSL::LinAlg

namespace NSL::Measure::Hubbard {

// k == q modulo the honeycomb reciprocal lattice (twoBodyCorrelationFunction.tpp:101-135).
inline bool eq_modBZ_gb300(double k0, double k1, double q0, double q1, double eps = 2e-12) {
    const double d0 = k0 - q0, d1 = k1 - q1;
    const double c0 = 4 * M_PI / 3, c1 = 0, e0 = -2 * M_PI / 3, e1 = 2 * M_PI / std::sqrt(3.0);
    const double den = c1 * e0 - c0 * e1;
    const double m = (d1 * e0 - d0 * e1) / den, n = (d0 * c1 - d1 * c0) / den;
    return std::abs(std::round(m) - m) < eps && std::abs(std::round(n) - n) < eps;
}

// TwoBodyCorrelator<Type, LatticeType, FermionMatrixType> (twoBodyCorrelationFunction.tpp:12-180) on libnslgpu,
// without the Measurement/HDF5 layer: constructed from (lattice, params) with params["Nt"], ["beta"], ["mu"],
// ["wallSources"] (nk, nb, Nx) and ["momenta"] (nk, 2); measure(phi, NumberTimeSources) evaluates one configuration
// (:188-306) and fills channel(c)[w][x][P][Q] with the reference's (Nt, nb^2, nb^2) tensors, c in the order of
// nslg_twobody_channel. The reference's file-level measure() reads phi from and writes these maps to its H5IO
// under "<basenode>/markovChain/<cfg>/correlators/twobody/<channel>/w-x-P-Q"; that loop stays with the caller.
template <NSL::Concept::isNumber Type, NSL::Concept::isDerived<NSL::Lattice::SpatialLattice<Type>> LatticeType,
          typename FermionMatrixType = NSL::FermionMatrix::HubbardExpGB300<Type, LatticeType>>
class TwoBodyCorrelatorGB300 {
  public:
    using map4D = std::unordered_map<
        NSL::size_t,
        std::unordered_map<NSL::size_t, std::unordered_map<NSL::size_t, std::unordered_map<NSL::size_t, NSL::Tensor<Type>>>>>;

    TwoBodyCorrelatorGB300(LatticeType &lattice, NSL::Parameter params, double eps = 1e-12,
                           NSL::size_t maxIter = 10000, int precision = NSLG_PREC_FP64)
        : hfm_(lattice, params), wall_(NSL::Tensor<Type>(params["wallSources"]), true), eps_(eps),
          maxIter_(maxIter), precision_(precision) {
        nk_ = wall_.shape(0);
        nb_ = wall_.shape(1);
        Nt_ = params["Nt"].template to<NSL::size_t>();
        NSL::Tensor<double> momenta = params["momenta"];
        for (NSL::size_t w = 0; w < nk_; ++w)
            for (NSL::size_t x = 0; x < nk_; ++x)
                for (NSL::size_t P = 0; P < nk_; ++P)
                    for (NSL::size_t Q = 0; Q < nk_; ++Q)
                        if (eq_modBZ_gb300(momenta(w, 0) + momenta(x, 0), momenta(w, 1) + momenta(x, 1),
                                           momenta(P, 0) + momenta(Q, 0), momenta(P, 1) + momenta(Q, 1)))
                            tuples_.insert(tuples_.end(), {int64_t(w), int64_t(x), int64_t(P), int64_t(Q)});
    }

    void measure(const NSL::Tensor<Type> &phi, NSL::size_t NumberTimeSources) {
        const int64_t nt = int64_t(tuples_.size() / 4), nb2 = nb_ * nb_;
        NSL::Tensor<Type> phic(phi, true);
        NSL::Tensor<Type> out(NSL::size_t(NSLG_TB_NCHANNELS), NSL::size_t(std::max<int64_t>(nt, 1)), Nt_, nb2, nb2);
        NSL::GB300::check(nslg_twobody_measure(hfm_.handle(), NSL::GB300::ptr(phic), NSL::GB300::ptr(wall_), nk_, nb_,
                                               tuples_.data(), nt, NumberTimeSources, eps_, maxIter_, precision_,
                                               NSL::GB300::ptr(out), &stats));
        for (int c = 0; c < NSLG_TB_NCHANNELS; ++c) {
            channels_[c].clear();
            for (int64_t u = 0; u < nt; ++u) {
                const int64_t *k = &tuples_[4 * u];
                channels_[c][k[0]][k[1]][k[2]][k[3]] = NSL::Tensor<Type>(out(c, u, NSL::Slice(), NSL::Slice(), NSL::Slice()), true);
            }
        }
    }

    const map4D &channel(int c) const { return channels_[c]; }
    nslg_cg_stats stats{};

  private:
    FermionMatrixType hfm_;
    NSL::Tensor<Type> wall_;
    double eps_;
    NSL::size_t maxIter_;
    int precision_;
    NSL::size_t nk_ = 0, nb_ = 0, Nt_ = 0;
    std::vector<int64_t> tuples_;
    map4D channels_[NSLG_TB_NCHANNELS];
};

// TwoPointCorrelator<Type, LatticeType, FermionMatrixType> (twoPointCorrelationFunction.tpp:17-109) on libnslgpu,
// without the Measurement/HDF5 layer: constructed from (lattice, params, species) with params["Nt"], ["beta"], ["mu"]
// and, for measureK, ["wallSources"] (nk, nb, Nx). measure(phi, NumberTimeSources) (:116-162) fills corr()
// (Nt, Nx, Nx) and measureK(phi, k, NumberTimeSources) (:169-233) fills corrKblock() (Nt, nb, nb), with the
// reference's source placement, shift t -> t - tsrc with the anti-periodic sign and division by NumberTimeSources.
// The reference runs one CG over the source batch per source time; here every source time's sources go into one
// solve of independent systems (NSLG_CG_PER_RHS, true-residual rule, eps per source: point and wall sources have
// unit norm) followed by one M^dagger application. A NumberTimeSources above Nt uses every time slice (the
// reference's integer step would be zero).
template <NSL::Concept::isNumber Type, NSL::Concept::isDerived<NSL::Lattice::SpatialLattice<Type>> LatticeType,
          typename FermionMatrixType = NSL::FermionMatrix::HubbardExpGB300<Type, LatticeType>>
class TwoPointCorrelatorGB300 {
  public:
    TwoPointCorrelatorGB300(LatticeType &lattice, NSL::Parameter params, NSL::Hubbard::Species species,
                            double eps = 1e-12, NSL::size_t maxIter = 10000, int precision = NSLG_PREC_FP64)
        : hfm_(lattice, params), species_(species), eps_(eps), maxIter_(maxIter), precision_(precision) {
        Nt_ = params["Nt"].template to<NSL::size_t>();
        Nx_ = lattice.sites();
        if (params.count("wallSources")) {
            wall_ = NSL::Tensor<Type>(NSL::Tensor<Type>(params["wallSources"]), true);
            nk_ = wall_.shape(0);
            nb_ = wall_.shape(1);
        }
    }

    void measure(const NSL::Tensor<Type> &phi, NSL::size_t NumberTimeSources) {
        const auto tsrcs = source_times_(NumberTimeSources);
        const NSL::size_t ns = tsrcs.size();
        hfm_.populate(phi, species_);
        NSL::Tensor<Type> src(phi.device(), ns, Nx_, Nt_, Nx_);
        for (NSL::size_t j = 0; j < ns; ++j)
            src.index_fill(Type(1), j, NSL::Range(Nx_), tsrcs[j], NSL::Range(Nx_));
        NSL::Tensor<Type> invM = solve_(src.reshape(ns * Nx_, Nt_, Nx_)).reshape(ns, Nx_, Nt_, Nx_);
        corr_ = NSL::Tensor<Type>(phi.device(), Nt_, Nx_, Nx_);
        for (NSL::size_t j = 0; j < ns; ++j) {
            NSL::Tensor<Type> blk(invM(j, NSL::Slice(), NSL::Slice(), NSL::Slice()), true);
            blk.shift(-tsrcs[j], -2, -Type(1));
            corr_ += blk.transpose(0, 1).transpose(1, 2);
        }
        corr_ /= Type(NumberTimeSources);
    }

    void measureK(const NSL::Tensor<Type> &phi, NSL::size_t k, NSL::size_t NumberTimeSources) {
        if (nb_ == 0 || k >= nk_) throw std::invalid_argument("TwoPointCorrelatorGB300::measureK: no wall source k");
        const auto tsrcs = source_times_(NumberTimeSources);
        const NSL::size_t ns = tsrcs.size();
        hfm_.populate(phi, species_);
        NSL::Tensor<Type> src(phi.device(), ns, nb_, Nt_, Nx_);
        for (NSL::size_t j = 0; j < ns; ++j)
            src(j, NSL::Slice(), tsrcs[j], NSL::Slice()) = wall_(k, NSL::Slice(), NSL::Slice());
        NSL::Tensor<Type> invM = solve_(src.reshape(ns * nb_, Nt_, Nx_)).reshape(ns, nb_, Nt_, Nx_);
        NSL::Tensor<Type> corrK(phi.device(), nb_, Nt_, Nx_);
        for (NSL::size_t j = 0; j < ns; ++j) {
            NSL::Tensor<Type> blk(invM(j, NSL::Slice(), NSL::Slice(), NSL::Slice()), true);
            corrK += blk.shift(-tsrcs[j], -2, -Type(1));
        }
        corrK /= Type(NumberTimeSources);
        corrKblock_ = NSL::Tensor<Type>(phi.device(), Nt_, nb_, nb_);
        for (NSL::size_t s1 = 0; s1 < nb_; ++s1) {
            NSL::Tensor<Type> w = NSL::Tensor<Type>(wall_(k, s1, NSL::Slice()), true).expand(Nt_, 0);
            for (NSL::size_t s2 = 0; s2 < nb_; ++s2)
                corrKblock_(NSL::Slice(), s1, s2) =
                    NSL::LinAlg::inner_product(w, NSL::Tensor<Type>(corrK(s2, NSL::Slice(), NSL::Slice())), 1);
        }
    }

    const NSL::Tensor<Type> &corr() const { return corr_; }
    const NSL::Tensor<Type> &corrKblock() const { return corrKblock_; }
    nslg_cg_stats stats{};

  private:
    std::vector<NSL::size_t> source_times_(NSL::size_t NumberTimeSources) const {
        if (NumberTimeSources <= 0) throw std::invalid_argument("TwoPointCorrelatorGB300: NumberTimeSources <= 0");
        const NSL::size_t step = std::max<NSL::size_t>(1, Nt_ / NumberTimeSources);
        std::vector<NSL::size_t> t;
        for (NSL::size_t tsrc = 0; tsrc < Nt_; tsrc += step) t.push_back(tsrc);
        return t;
    }

    // M^{-1} b = M^dagger (M M^dagger)^{-1} b for every (Nt, Nx) source in b
    NSL::Tensor<Type> solve_(const NSL::Tensor<Type> &b) {
        NSL::Tensor<Type> bb(b, true), x(b, true);
        const int64_t nbatch = bb.numel() / (Nt_ * Nx_);
        NSL::GB300::check(nslg_cg_solve(hfm_.handle(), NSLG_OP_MMDAGGER, NSL::GB300::ptr(bb), nullptr,
                                        NSL::GB300::ptr(x), nbatch, eps_, maxIter_, NSLG_CG_PER_RHS, precision_,
                                        NSLG_STOP_TRUE_RESIDUAL, &stats));
        return hfm_.Mdagger(x);
    }

    FermionMatrixType hfm_;
    NSL::Hubbard::Species species_;
    double eps_;
    NSL::size_t maxIter_;
    int precision_;
    NSL::size_t Nt_ = 0, Nx_ = 0, nk_ = 0, nb_ = 0;
    NSL::Tensor<Type> wall_, corr_, corrKblock_;
};

}  // namespace NSL::Measure::Hubbard
