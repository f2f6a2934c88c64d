// Host-side run of the C++ drop-in classes (include/nsl_gb300/nsl_dropin.hpp) on the CPU. Test infrastructure (built
// and run by tests/test_dropin_cpp.py where the reference checkout is present). Built with -DNSLG_DROPIN_DEVICE
// and linked to libnslgpu.so instead, the same drivers run the classes on the GPU through the real library
// (tests/test_gpu_dropin_cpp.py).
//
// The libnslgpu entry points the classes reach are replaced by a host stand-in over the reference's own HubbardExp
// and CG (hubbardExp.tpp, CG.tpp): nslg_fm_apply, nslg_fm_logdet and nslg_fm_grad_logdet call the reference
// operators, nslg_cg_solve runs the reference CG one right-hand side at a time (as NSLG_CG_PER_RHS does). The outputs
// are compared with the reference's own outputs in the golden fixtures, so this checks the drop-in's own steps: the
// two-point correlator's source placement, shifts, averaging and projection, and HubbardExpGB300 running inside the
// reference's HubbardFermionAction, Action sum, Leapfrog and LeapfrogRealForce templates (copies, populate order).
//
// Usage: dropin_host <case-dir> twopoint, with params.txt "L1 L2 Nt beta mu nk nb nts", phi.bin (Nt, Nx) and
// wall.bin (nk, nb, Nx) as raw complex128; writes corr_P.bin, corr_H.bin (Nt, Nx, Nx), block_P.bin, block_H.bin
// (nk, Nt, nb, nb). Or dropin_host <case-dir> action, with params.txt "L1 L2 Nt beta mu U nmd tau", phi.bin and
// p.bin (Nt, Nx); writes S.bin, force.bin, lf_q.bin, lf_p.bin, lfr_q.bin, lfr_p.bin. Or dropin_host <case-dir> cg,
// with params.txt "L1 L2 Nt beta mu eps maxIter R", phi.bin and b.bin (R, Nt, Nx); writes cg_x.bin.
#include "nsl_shims.hpp"

#include <cstdio>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

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

namespace {
Lat *g_lattice = nullptr;  // the lattice the stand-in fermion matrices are built on
std::string g_error;
}  // namespace

#ifndef NSLG_DROPIN_DEVICE
struct nslg_ctx {
    int device;
};
struct nslg_fm {
    std::unique_ptr<NSL::FermionMatrix::HubbardExp<C, Lat>> hfm;
    int64_t Nt, Nx;
    int species;
};

namespace {
NSL::Tensor<C> wrap(const nslg_c128 *p, int64_t nbatch, int64_t Nt, int64_t Nx) {
    auto t = torch::from_blob(const_cast<nslg_c128 *>(p), {nbatch, Nt, Nx}, torch::kComplexDouble);
    return NSL::Tensor<C>(t.clone());
}
void store(const NSL::Tensor<C> &t, nslg_c128 *out) {
    auto c = torch::Tensor(t).contiguous();
    std::memcpy(out, c.data_ptr(), c.numel() * sizeof(nslg_c128));
}
}  // namespace

extern "C" {
const char *nslg_last_error(void) { return g_error.c_str(); }
int nslg_ctx_create(int device, void *, nslg_ctx **out) {
    *out = new nslg_ctx{device};
    return NSLG_OK;
}
int nslg_fm_create_kind(nslg_ctx *, int kind, int64_t Nx, int64_t Nt, const nslg_c128 *, nslg_c128 beta, nslg_c128 mu,
                        int species, nslg_fm **out) {
    if (kind != NSLG_FM_EXP || !g_lattice || g_lattice->sites() != Nx) return NSLG_ERR_UNSUPPORTED;
    auto *fm = new nslg_fm{nullptr, Nt, Nx, species};
    fm->hfm = std::make_unique<NSL::FermionMatrix::HubbardExp<C, Lat>>(*g_lattice, Nt, C(beta.re, beta.im),
                                                                       C(mu.re, mu.im));
    *out = fm;
    return NSLG_OK;
}
int nslg_fm_destroy(nslg_fm *fm) {
    delete fm;
    return NSLG_OK;
}
int nslg_fm_set_exp_hopping(nslg_fm *, nslg_c128, const nslg_c128 *) { return NSLG_OK; }
int nslg_fm_populate(nslg_fm *fm, const nslg_c128 *phi, int species) {
    if (species >= 0) fm->species = species;
    NSL::Tensor<C> p(torch::Tensor(wrap(phi, 1, fm->Nt, fm->Nx)).select(0, 0).contiguous());
    fm->hfm->populate(p, fm->species == NSLG_PARTICLE ? NSL::Hubbard::Particle : NSL::Hubbard::Hole);
    return NSLG_OK;
}
int nslg_fm_apply(nslg_fm *fm, int op, const nslg_c128 *psi, nslg_c128 *out, int64_t nbatch, int) {
    NSL::Tensor<C> v = wrap(psi, nbatch, fm->Nt, fm->Nx);
    switch (op) {
    case NSLG_OP_M: store(fm->hfm->M(v), out); break;
    case NSLG_OP_MDAGGER: store(fm->hfm->Mdagger(v), out); break;
    case NSLG_OP_MMDAGGER: store(fm->hfm->MMdagger(v), out); break;
    case NSLG_OP_MDAGGERM: store(fm->hfm->MdaggerM(v), out); break;
    default: return NSLG_ERR_ARG;
    }
    return NSLG_OK;
}
int nslg_cg_solve(nslg_fm *fm, int op, const nslg_c128 *b, const nslg_c128 *x0, nslg_c128 *x, int64_t nbatch,
                  double eps, int64_t max_iter, int mode, int, int, nslg_cg_stats *stats) {
    if (op != NSLG_OP_MMDAGGER || x0) return NSLG_ERR_UNSUPPORTED;
    const int64_t n = fm->Nt * fm->Nx;
    if (mode == NSLG_CG_SHARED) {  // the reference's own solve of the whole batch
        NSL::LinAlg::CG<C> cg(*fm->hfm, NSL::FermionMatrix::MMdagger, eps, max_iter);
        store(cg(wrap(b, nbatch, fm->Nt, fm->Nx)), x);
        if (stats) *stats = nslg_cg_stats{0, 0, 1, 1, 0.0, 0.0, 0};
        return NSLG_OK;
    }
    if (mode != NSLG_CG_PER_RHS) return NSLG_ERR_ARG;
    for (int64_t i = 0; i < nbatch; ++i) {
        NSL::LinAlg::CG<C> cg(*fm->hfm, NSL::FermionMatrix::MMdagger, 1e-14, 100000);
        NSL::Tensor<C> bi(torch::Tensor(wrap(b + i * n, 1, fm->Nt, fm->Nx)).select(0, 0).contiguous());
        store(cg(bi), x + i * n);
    }
    if (stats) *stats = nslg_cg_stats{0, 0, nbatch, nbatch, 0.0, 0.0, 0};
    return NSLG_OK;
}
int nslg_fm_logdet(nslg_fm *fm, nslg_c128 *out) {
    const C ld = fm->hfm->logDetM();
    *out = nslg_c128{ld.real(), ld.imag()};
    return NSLG_OK;
}
int nslg_fm_grad_logdet(nslg_fm *fm, nslg_c128 *out) {
    store(fm->hfm->gradLogDetM(), out);
    return NSLG_OK;
}
}
#endif  // NSLG_DROPIN_DEVICE

namespace {

NSL::Tensor<C> read_c128(const std::string &path, std::vector<int64_t> shape) {
    int64_t n = 1;
    for (auto s : shape) n *= s;
    std::vector<nslg_c128> buf(n);
    std::FILE *f = std::fopen(path.c_str(), "rb");
    if (!f || std::fread(buf.data(), sizeof(nslg_c128), n, f) != size_t(n)) throw std::runtime_error(path);
    std::fclose(f);
    return NSL::Tensor<C>(torch::from_blob(buf.data(), shape, torch::kComplexDouble).clone());
}

void write_c128(const std::string &path, const NSL::Tensor<C> &t) {
    auto c = torch::Tensor(t).contiguous();
    std::FILE *f = std::fopen(path.c_str(), "wb");
    std::fwrite(c.data_ptr(), sizeof(nslg_c128), c.numel(), f);
    std::fclose(f);
}

void write_scalar(const std::string &path, const C &v) {
    NSL::Tensor<C> t(1);
    t(0) = v;
    write_c128(path, t);
}

const std::pair<NSL::Hubbard::Species, const char *> kSpecies[] = {{NSL::Hubbard::Particle, "P"},
                                                                   {NSL::Hubbard::Hole, "H"}};

int run_twopoint(const std::string &dir) {
    std::ifstream in(dir + "/params.txt");
    int L1, L2;
    int64_t Nt, nk, nb, nts;
    double beta, mu;
    in >> L1 >> L2 >> Nt >> beta >> mu >> nk >> nb >> nts;
    Lat lat(std::vector<int>{L1, L2});
    g_lattice = &lat;
    const int64_t Nx = lat.sites();
    NSL::Parameter params;
    params["beta"] = C(beta);
    params["mu"] = C(mu);
    params["Nt"] = Nt;
    params["Nx"] = Nx;
    params["wallSources"] = read_c128(dir + "/wall.bin", {nk, nb, Nx});
    const NSL::Tensor<C> phi = read_c128(dir + "/phi.bin", {Nt, Nx});
    for (auto [sp, tag] : kSpecies) {
        NSL::Measure::Hubbard::TwoPointCorrelatorGB300<C, Lat> tp(lat, params, sp);
        tp.measure(phi, nts);
        write_c128(dir + "/corr_" + tag + ".bin", tp.corr());
        std::vector<torch::Tensor> blocks;
        for (int64_t k = 0; k < nk; ++k) {
            tp.measureK(phi, k, nts);
            blocks.push_back(torch::Tensor(tp.corrKblock()).clone());
        }
        write_c128(dir + "/block_" + tag + ".bin", NSL::Tensor<C>(torch::stack(blocks)));
    }
    return 0;
}

// HubbardExpGB300 in the template slots the reference's own HMC code uses (hubbardFermiAction.tpp, leapfrog.tpp).
int run_action(const std::string &dir) {
    std::ifstream in(dir + "/params.txt");
    int L1, L2;
    int64_t Nt, Nmd;
    double beta, mu, U, tau;
    in >> L1 >> L2 >> Nt >> beta >> mu >> U >> Nmd >> tau;
    Lat lat(std::vector<int>{L1, L2});
    g_lattice = &lat;
    const int64_t Nx = lat.sites();
    NSL::Parameter params;
    params["beta"] = C(beta);
    params["U"] = C(U);
    params["mu"] = C(mu);
    params["Nt"] = Nt;
    using HFM = NSL::FermionMatrix::HubbardExpGB300<C, Lat>;
    NSL::Action::HubbardGaugeAction<C> S_gauge(params);
    NSL::Action::HubbardFermionAction<C, Lat, HFM> S_fermion(lat, params);
    NSL::Action::Action S = S_gauge + S_fermion;
    NSL::Configuration<C> q{{"phi", read_c128(dir + "/phi.bin", {Nt, Nx})}};
    NSL::Configuration<C> p{{"phi", read_c128(dir + "/p.bin", {Nt, Nx})}};
    write_scalar(dir + "/S.bin", S(q));
    write_c128(dir + "/force.bin", S.force(q)["phi"]);
    NSL::Integrator::Leapfrog lf(S, tau, Nmd);
    auto [q1, p1] = lf(q, p);
    write_c128(dir + "/lf_q.bin", q1["phi"]);
    write_c128(dir + "/lf_p.bin", p1["phi"]);
    NSL::Integrator::LeapfrogRealForce lfr(S, tau, Nmd);
    auto [q2, p2] = lfr(q, p);
    write_c128(dir + "/lfr_q.bin", q2["phi"]);
    write_c128(dir + "/lfr_p.bin", p2["phi"]);
    return 0;
}

// CGGB300 on MM^dagger for the particle species (CG.hpp:142-186 semantics through nslg_cg_solve, NSLG_CG_SHARED).
int run_cg(const std::string &dir) {
    std::ifstream in(dir + "/params.txt");
    int L1, L2;
    int64_t Nt, R, maxIter;
    double beta, mu, eps;
    in >> L1 >> L2 >> Nt >> beta >> mu >> eps >> maxIter >> R;
    Lat lat(std::vector<int>{L1, L2});
    g_lattice = &lat;
    const int64_t Nx = lat.sites();
    NSL::FermionMatrix::HubbardExpGB300<C, Lat> hfm(lat, Nt, C(beta), C(mu));
    hfm.populate(read_c128(dir + "/phi.bin", {Nt, Nx}), NSL::Hubbard::Particle);
    NSL::LinAlg::CGGB300<C> cg(hfm, NSL::FermionMatrix::MMdagger, eps, maxIter);
    write_c128(dir + "/cg_x.bin", cg(read_c128(dir + "/b.bin", {R, Nt, Nx})));
    return 0;
}

}  // namespace

int main(int argc, char **argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s <case-dir> twopoint|action|cg\n", argv[0]);
        return 2;
    }
    torch::set_num_threads(1);
    const std::string mode = argv[2];
    if (mode == "twopoint") return run_twopoint(argv[1]);
    if (mode == "action") return run_action(argv[1]);
    if (mode == "cg") return run_cg(argv[1]);
    std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
    return 2;
}
