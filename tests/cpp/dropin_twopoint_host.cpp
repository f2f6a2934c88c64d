// Host-side check of TwoPointCorrelatorGB300 (include/nsl_gb300/nsl_dropin.hpp): its source placement, source-time
// shifts, averaging and momentum projection, run on the CPU. Test infrastructure (built and run by
// tests/test_dropin_cpp.py where the reference checkout is present).
//
// The libnslgpu entry points the class reaches are replaced by a host stand-in over the reference's own HubbardExp
// and CG (hubbardExp.tpp, CG.tpp): nslg_fm_apply applies the reference operators, nslg_cg_solve runs the reference CG
// one right-hand side at a time (as NSLG_CG_PER_RHS does). The outputs are compared with the reference's
// TwoPointCorrelator outputs in the golden fixtures, so this checks the drop-in's own tensor steps.
//
// Usage: dropin_twopoint_host <case-dir> with params.txt ("L1 L2 Nt beta mu nk nb nts"), phi.bin (Nt, Nx) and
// wall.bin (nk, nb, Nx) as raw complex128; writes corr_P.bin, corr_H.bin (Nt, Nx, Nx), block_P.bin, block_H.bin
// (nk, Nt, nb, nb).
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

#include "nsl_gb300/nsl_dropin.hpp"

using C = NSL::complex<double>;
using Lat = NSL::Lattice::Honeycomb<C>;

namespace {
Lat *g_lattice = nullptr;  // the lattice the stand-in fermion matrices are built on
std::string g_error;
}  // namespace

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
int nslg_cg_solve(nslg_fm *fm, int op, const nslg_c128 *b, const nslg_c128 *, nslg_c128 *x, int64_t nbatch, double,
                  int64_t, int mode, int, int, nslg_cg_stats *stats) {
    if (op != NSLG_OP_MMDAGGER || mode != NSLG_CG_PER_RHS) return NSLG_ERR_UNSUPPORTED;
    const int64_t n = fm->Nt * fm->Nx;
    for (int64_t i = 0; i < nbatch; ++i) {
        NSL::LinAlg::CG<C> cg(*fm->hfm, NSL::FermionMatrix::MMdagger, 1e-14, 100000);
        NSL::Tensor<C> bi(torch::Tensor(wrap(b + i * n, 1, fm->Nt, fm->Nx)).select(0, 0).contiguous());
        store(cg(bi), x + i * n);
    }
    if (stats) *stats = nslg_cg_stats{0, 0, nbatch, nbatch, 0.0, 0.0, 0};
    return NSLG_OK;
}
int nslg_fm_logdet(nslg_fm *, nslg_c128 *) { return NSLG_ERR_UNSUPPORTED; }
int nslg_fm_grad_logdet(nslg_fm *, nslg_c128 *) { return NSLG_ERR_UNSUPPORTED; }
}

int main(int argc, char **argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: %s <case-dir>\n", argv[0]);
        return 2;
    }
    torch::set_num_threads(1);
    const std::string dir = argv[1];
    std::ifstream in(dir + "/params.txt");
    int L1, L2;
    int64_t Nt, nk, nb, nts;
    double beta, mu;
    in >> L1 >> L2 >> Nt >> beta >> mu >> nk >> nb >> nts;
    Lat lat(std::vector<int>{L1, L2});
    g_lattice = &lat;
    const int64_t Nx = lat.sites();
    auto read = [&](const std::string &name, std::vector<int64_t> shape) {
        int64_t n = 1;
        for (auto s : shape) n *= s;
        std::vector<nslg_c128> buf(n);
        std::FILE *f = std::fopen((dir + "/" + name).c_str(), "rb");
        if (!f || std::fread(buf.data(), sizeof(nslg_c128), n, f) != size_t(n)) throw std::runtime_error(name);
        std::fclose(f);
        return NSL::Tensor<C>(torch::from_blob(buf.data(), shape, torch::kComplexDouble).clone());
    };
    auto write = [&](const std::string &name, const NSL::Tensor<C> &t) {
        auto c = torch::Tensor(t).contiguous();
        std::FILE *f = std::fopen((dir + "/" + name).c_str(), "wb");
        std::fwrite(c.data_ptr(), sizeof(nslg_c128), c.numel(), f);
        std::fclose(f);
    };
    NSL::Parameter params;
    params["beta"] = C(beta);
    params["mu"] = C(mu);
    params["Nt"] = Nt;
    params["Nx"] = Nx;
    params["wallSources"] = read("wall.bin", {nk, nb, Nx});
    const NSL::Tensor<C> phi = read("phi.bin", {Nt, Nx});
    const std::pair<NSL::Hubbard::Species, const char *> species[] = {{NSL::Hubbard::Particle, "P"},
                                                                      {NSL::Hubbard::Hole, "H"}};
    for (auto [sp, tag] : species) {
        NSL::Measure::Hubbard::TwoPointCorrelatorGB300<C, Lat> tp(lat, params, sp);
        tp.measure(phi, nts);
        write(std::string("corr_") + tag + ".bin", tp.corr());
        std::vector<torch::Tensor> blocks;
        for (int64_t k = 0; k < nk; ++k) {
            tp.measureK(phi, k, nts);
            blocks.push_back(torch::Tensor(tp.corrKblock()).clone());
        }
        write(std::string("block_") + tag + ".bin", NSL::Tensor<C>(torch::stack(blocks)));
    }
    return 0;
}
