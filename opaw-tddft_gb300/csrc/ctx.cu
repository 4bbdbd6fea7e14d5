// ctx.cu — context lifetime, operator-table upload and the C ABI entry points
// for state and per-routine operators (include/opaw_gb300.h).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "fft.cuh"

namespace opaw {

static thread_local std::string g_err;
void set_error(const std::string &msg) { g_err = msg; }
const char *get_error() { return g_err.c_str(); }

int ensure(DeviceBuf &b, size_t bytes) {
  if (b.bytes >= bytes && b.p) return OPAW_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  cudaError_t e = cudaMalloc(&b.p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    set_error(std::string("device allocation of ") + std::to_string(bytes) + " bytes: " + cudaGetErrorString(e));
    b.p = nullptr;
    return OPAW_ERR_NOMEM;
  }
  b.bytes = bytes;
  return OPAW_OK;
}

template <typename T> static int upload(T **dst, const T *src, size_t n) {
  OPAW_CUDA(cudaMalloc((void **)dst, sizeof(T) * (n ? n : 1)));
  if (n && src) OPAW_CUDA(cudaMemcpy(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice));
  else OPAW_CUDA(cudaMemset(*dst, 0, sizeof(T) * (n ? n : 1)));
  return OPAW_OK;
}

// k component of grid index i on an axis of n points, spacing d (ek.f90:18-32)
static double kcomp(int i, int n, double d) {
  const double pi = acos(-1.0);
  double dk = 2.0 * pi / (n * d);
  double k = (double)i * dk;
  if (k > pi / d) k = k - 2.0 * pi / d;
  return k;
}

int vk_prep(opaw_ctx *c);  // rebuild.cu

static int build(opaw_ctx *c, const opaw_system *s) {
  c->nx = s->nx;
  c->ny = s->ny;
  c->nz = s->nz;
  c->nn = (int64_t)s->nx * s->ny * s->nz;
  c->dx = s->dx;
  c->dy = s->dy;
  c->dz = s->dz;
  c->dv = s->dx * s->dy * s->dz;
  c->ekcut = s->ekcut;
  c->rnel = s->rnel;
  c->dij_max = s->dij_max;
  c->periodic = s->periodic;
  c->scale_vh = s->scale_vh > 0 ? s->scale_vh : 1;
  c->nxb = c->scale_vh * c->nx;
  c->nyb = c->scale_vh * c->ny;
  c->nzb = c->scale_vh * c->nz;
  c->nnb = (int64_t)c->nxb * c->nyb * c->nzb;
  c->natom = s->natom;
  OPAW_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  OPAW_CUDA(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
  OPAW_CUDA(cudaEventCreateWithFlags(&c->side_fork, cudaEventDisableTiming));
  OPAW_CUDA(cudaEventCreateWithFlags(&c->side_join, cudaEventDisableTiming));
  OPAW_CUDA(cudaMalloc(&c->d_tma_err, sizeof(int)));
  OPAW_CUDA(cudaMemset(c->d_tma_err, 0, sizeof(int)));
  {
    int dev = 0;
    OPAW_CUDA(cudaGetDevice(&dev));
    OPAW_CUDA(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, dev));
  }

  const int na = s->natom;
  c->h_ms.assign(s->ms, s->ms + na);
  c->h_nrough.assign(s->nrough, s->nrough + 3 * na);
  c->h_ir0.resize(3 * na);
  c->h_poff.assign(na + 1, 0);
  c->h_soff.assign(na + 1, 0);
  c->h_doff.assign(na + 1, 0);
  c->msmax = 0;
  const int nd3[3] = {c->nx, c->ny, c->nz};
  for (int a = 0; a < na; a++) {
    const int m = s->ms[a];
    OPAW_ARG(m > 0 && m <= 16, "projectors per atom must be in [1, 16]");
    int64_t nbox = 1;
    for (int k = 0; k < 3; k++) {
      const int nr = s->nrough[3 * a + k];
      OPAW_ARG(nr > 0 && nr <= nd3[k], "projector box larger than the grid (read_paw.f90:254)");
      const int i0 = s->ir_start[3 * a + k] - 1;
      if (!s->periodic && (i0 < 0 || i0 + nr > nd3[k])) {
        set_error("non periodic, local grid cannot go outside box: atom " + std::to_string(a + 1));
        return OPAW_ERR_BOX;  // get_irs.f90:30-35
      }
      OPAW_ARG(i0 > -nd3[k] && i0 < nd3[k], "box origin more than one period outside the grid");
      c->h_ir0[3 * a + k] = i0;
      nbox *= nr;
    }
    c->maxbox = std::max(c->maxbox, (int)nbox);
    c->msmax = std::max(c->msmax, m);
    c->h_poff[a + 1] = c->h_poff[a] + m * nbox;
    c->h_soff[a + 1] = c->h_soff[a] + m;
    c->h_doff[a + 1] = c->h_doff[a] + (int64_t)m * m;
  }
  c->ns = (int)c->h_soff[na];
  c->nd = (int)c->h_doff[na];
  const int64_t np = c->h_poff[na];
  OPAW_CHECK(upload(&c->d_ms, s->ms, na));
  OPAW_CHECK(upload(&c->d_nrough, s->nrough, 3 * na));
  OPAW_CHECK(upload(&c->d_ir0, c->h_ir0.data(), 3 * na));
  OPAW_CHECK(upload(&c->d_poff, c->h_poff.data(), na + 1));
  OPAW_CHECK(upload(&c->d_soff, c->h_soff.data(), na + 1));
  OPAW_CHECK(upload(&c->d_doff, c->h_doff.data(), na + 1));
  OPAW_CHECK(upload(&c->d_p3d, s->p3d, np));
  OPAW_CHECK(upload(&c->d_p3d1, s->p3d1, np));
  {
    std::vector<float> f(np);
    for (int64_t i = 0; i < np; i++) f[i] = (float)s->p3d[i];
    OPAW_CHECK(upload(&c->d_p3d_f, f.data(), np));
    for (int64_t i = 0; i < np; i++) f[i] = (float)s->p3d1[i];
    OPAW_CHECK(upload(&c->d_p3d1_f, f.data(), np));
  }
  OPAW_CHECK(upload(&c->d_s, s->s, c->ns));
  OPAW_CHECK(upload(&c->d_sinv, s->sinv, c->ns));
  {
    const double ns_[4] = {-1.0, -0.5, 0.5, 1.0};
    std::vector<double> sg(c->ns);
    for (int k = 0; k < 4; k++) {
      for (int t = 0; t < c->ns; t++)
        sg[t] = (k == 0) ? s->sinv[t] : pow(1.0 + s->s[t], ns_[k]) - 1.0;  // snphi.f90:24-28
      OPAW_CHECK(upload(&c->d_sigma[k], sg.data(), c->ns));
    }
    std::vector<int> sa(c->ns), da(c->nd);
    for (int a = 0; a < na; a++) {
      for (int64_t t = c->h_soff[a]; t < c->h_soff[a + 1]; t++) sa[t] = a;
      for (int64_t t = c->h_doff[a]; t < c->h_doff[a + 1]; t++) da[t] = a;
    }
    OPAW_CHECK(upload(&c->d_slot_atom, sa.data(), c->ns));
    OPAW_CHECK(upload(&c->d_dslot_atom, da.data(), c->nd));
  }
  // union of projector boxes as CSR over grid points, atoms ascending
  {
    struct Ent { int64_t g; int a; int b; };
    std::vector<Ent> ents;
    for (int a = 0; a < na; a++) {
      const int n0 = s->nrough[3 * a], n1 = s->nrough[3 * a + 1], n2 = s->nrough[3 * a + 2];
      int b = 0;
      for (int bz = 0; bz < n2; bz++)
        for (int by = 0; by < n1; by++)
          for (int bx = 0; bx < n0; bx++, b++) {
            int ix = (c->h_ir0[3 * a] + bx + c->nx) % c->nx;
            int iy = (c->h_ir0[3 * a + 1] + by + c->ny) % c->ny;
            int iz = (c->h_ir0[3 * a + 2] + bz + c->nz) % c->nz;
            ents.push_back({ix + (int64_t)c->nx * (iy + (int64_t)c->ny * iz), a, b});
          }
    }
    std::stable_sort(ents.begin(), ents.end(), [](const Ent &x, const Ent &y) { return x.g < y.g; });
    std::vector<int> boxg(ents.size());
    std::vector<int64_t> boff(na + 1, 0);
    for (int a = 0; a < na; a++)
      boff[a + 1] = boff[a] + (int64_t)s->nrough[3 * a] * s->nrough[3 * a + 1] * s->nrough[3 * a + 2];
    for (const Ent &e : ents) boxg[boff[e.a] + e.b] = (int)e.g;
    OPAW_CHECK(upload(&c->d_boxg, boxg.data(), boxg.size()));
    OPAW_CHECK(upload(&c->d_boff, boff.data(), boff.size()));
    std::vector<int> upt, ustart, uatom, ubox;
    for (size_t i = 0; i < ents.size(); i++) {
      if (i == 0 || ents[i].g != ents[i - 1].g) {
        upt.push_back((int)ents[i].g);
        ustart.push_back((int)i);
      }
      uatom.push_back(ents[i].a);
      ubox.push_back(ents[i].b);
    }
    ustart.push_back((int)ents.size());
    c->nunion = (int)upt.size();
    c->nuent = (int)ents.size();
    OPAW_CHECK(upload(&c->d_upt, upt.data(), upt.size()));
    OPAW_CHECK(upload(&c->d_ustart, ustart.data(), ustart.size()));
    OPAW_CHECK(upload(&c->d_uatom, uatom.data(), uatom.size()));
    OPAW_CHECK(upload(&c->d_ubox, ubox.data(), ubox.size()));
    if (c->h_poff[na] < INT32_MAX) {
      // distinct atoms of every tile of kUTile union points, in order of
      // first appearance, and each entry's index among them
      const int nu = (int)upt.size(), ntile = (nu + kUTile - 1) / kUTile;
      std::vector<int4> uent(ents.size());
      std::vector<std::vector<int>> tat(ntile);
      for (int u = 0; u < nu; u++) {
        std::vector<int> &ta = tat[u / kUTile];
        for (int e = ustart[u]; e < ustart[u + 1]; e++) {
          const int a = ents[e].a;
          int la = (int)(std::find(ta.begin(), ta.end(), a) - ta.begin());
          if (la == (int)ta.size()) ta.push_back(a);
          const int nbox = s->nrough[3 * a] * s->nrough[3 * a + 1] * s->nrough[3 * a + 2];
          uent[e] = make_int4((int)(c->h_poff[a] + ents[e].b), la, s->ms[a], nbox);
        }
      }
      int amax = 1;
      for (const auto &ta : tat) amax = std::max(amax, (int)ta.size());
      std::vector<int2> ut((size_t)ntile * amax, make_int2(0, 0));
      std::vector<int> utn(ntile);
      for (int t = 0; t < ntile; t++) {
        utn[t] = (int)tat[t].size();
        for (int k = 0; k < utn[t]; k++) ut[(size_t)t * amax + k] = make_int2((int)c->h_soff[tat[t][k]], s->ms[tat[t][k]]);
      }
      c->uamax = amax;
      OPAW_CHECK(upload(&c->d_uent, uent.data(), uent.size()));
      OPAW_CHECK(upload(&c->d_utile, ut.data(), ut.size()));
      OPAW_CHECK(upload(&c->d_utile_na, utn.data(), utn.size()));
    }
    std::vector<int> uidx((size_t)c->nn, -1);
    for (int u = 0; u < c->nunion; u++) uidx[upt[u]] = u;
    OPAW_CHECK(upload(&c->d_uidx, uidx.data(), uidx.size()));
    // projector overlaps: every pair of entries at a union point adds
    // P_x[a][i](b) P_y[a'][j](b') dv to block (a, a'), element (i, j)
    std::vector<std::vector<int>> nbr(na);
    for (int u = 0; u < c->nunion; u++)
      for (int e1 = ustart[u]; e1 < ustart[u + 1]; e1++)
        for (int e2 = ustart[u]; e2 < ustart[u + 1]; e2++) nbr[uatom[e1]].push_back(uatom[e2]);
    std::vector<int> ostart(na + 1, 0), oatom;
    std::vector<int64_t> ooff;
    int64_t tot = 0;
    for (int a = 0; a < na; a++) {
      std::sort(nbr[a].begin(), nbr[a].end());
      nbr[a].erase(std::unique(nbr[a].begin(), nbr[a].end()), nbr[a].end());
      for (int b : nbr[a]) {
        oatom.push_back(b);
        ooff.push_back(tot);
        tot += (int64_t)s->ms[a] * s->ms[b];
      }
      ostart[a + 1] = (int)oatom.size();
    }
    c->novl = (int)oatom.size();
    auto block_of = [&](int a, int b) {
      const int k0 = ostart[a], k1 = ostart[a + 1];
      const int k = (int)(std::lower_bound(oatom.begin() + k0, oatom.begin() + k1, b) - oatom.begin());
      return k;
    };
    std::vector<double> ov[4];
    for (auto &v : ov) v.assign((size_t)(tot ? tot : 1), 0.0);
    const double *tab[2] = {s->p3d, s->p3d1};
    for (int u = 0; u < c->nunion; u++)
      for (int e1 = ustart[u]; e1 < ustart[u + 1]; e1++) {
        const int a = uatom[e1], ba = ubox[e1], ma = s->ms[a];
        const int64_t na_box = boff[a + 1] - boff[a];
        for (int e2 = ustart[u]; e2 < ustart[u + 1]; e2++) {
          const int b = uatom[e2], bb = ubox[e2], mb = s->ms[b];
          const int64_t nb_box = boff[b + 1] - boff[b];
          const int64_t off = ooff[block_of(a, b)];
          for (int x = 0; x < 2; x++)
            for (int y = 0; y < 2; y++) {
              double *O = ov[2 * x + y].data() + off;
              for (int i = 0; i < ma; i++) {
                const double pa = tab[x][c->h_poff[a] + (int64_t)i * na_box + ba] * c->dv;
                for (int j = 0; j < mb; j++) O[(int64_t)i * mb + j] += pa * tab[y][c->h_poff[b] + (int64_t)j * nb_box + bb];
              }
            }
        }
      }
    OPAW_CHECK(upload(&c->d_ovl_start, ostart.data(), ostart.size()));
    OPAW_CHECK(upload(&c->d_ovl_atom, oatom.data(), oatom.size()));
    OPAW_CHECK(upload(&c->d_ovl_off, ooff.data(), ooff.size()));
    for (int k = 0; k < 4; k++) OPAW_CHECK(upload(&c->d_ovl[k], ov[k].data(), ov[k].size()));
  }
  // compensation spheres
  c->h_ngrid.assign(s->ngrid, s->ngrid + na);
  c->h_nlm.assign(s->nlm, s->nlm + na);
  c->h_goff.assign(na + 1, 0);
  c->h_g3off.assign(na + 1, 0);
  c->h_qoff.assign(na + 1, 0);
  c->h_eoff.assign(na + 1, 0);
  c->nlmmax = 0;
  for (int a = 0; a < na; a++) {
    const int64_t m = s->ms[a];
    OPAW_ARG(s->ngrid[a] >= 0 && s->nlm[a] >= 0 && s->nlm[a] <= 64, "bad compensation-sphere sizes");
    c->nlmmax = std::max(c->nlmmax, s->nlm[a]);
    c->h_goff[a + 1] = c->h_goff[a] + s->ngrid[a];
    c->h_g3off[a + 1] = c->h_g3off[a] + (int64_t)s->ngrid[a] * s->nlm[a];
    c->h_qoff[a + 1] = c->h_qoff[a] + (int64_t)s->nlm[a] * m * m;
    c->h_eoff[a + 1] = c->h_eoff[a] + m * m * m * m;
  }
  c->ncomp = (int)c->h_goff[na];
  {
    std::vector<int> gpt(c->ncomp);
    struct Ent { int g; int a; int ig; };
    std::vector<Ent> ents;
    for (int a = 0; a < na; a++)
      for (int ig = 0; ig < s->ngrid[a]; ig++) {
        const int *lg = s->local_grid + 3 * (c->h_goff[a] + ig);
        const int ix = lg[0] - 1, iy = lg[1] - 1, iz = lg[2] - 1;
        OPAW_ARG(ix >= 0 && ix < c->nx && iy >= 0 && iy < c->ny && iz >= 0 && iz < c->nz,
                 "compensation-sphere point outside the grid");
        const int g = ix + c->nx * (iy + c->ny * iz);
        gpt[c->h_goff[a] + ig] = g;
        ents.push_back({g, a, ig});
      }
    std::stable_sort(ents.begin(), ents.end(), [](const Ent &x, const Ent &y) { return x.g < y.g; });
    std::vector<int> cpt, cstart, catom, cig;
    for (size_t i = 0; i < ents.size(); i++) {
      if (i == 0 || ents[i].g != ents[i - 1].g) {
        cpt.push_back(ents[i].g);
        cstart.push_back((int)i);
      }
      catom.push_back(ents[i].a);
      cig.push_back(ents[i].ig);
    }
    cstart.push_back((int)ents.size());
    c->ncunion = (int)cpt.size();
    OPAW_CHECK(upload(&c->d_gpt, gpt.data(), gpt.size()));
    OPAW_CHECK(upload(&c->d_cpt, cpt.data(), cpt.size()));
    OPAW_CHECK(upload(&c->d_cstart, cstart.data(), cstart.size()));
    OPAW_CHECK(upload(&c->d_catom, catom.data(), catom.size()));
    OPAW_CHECK(upload(&c->d_cig, cig.data(), cig.size()));
  }
  OPAW_CHECK(upload(&c->d_ngrid, s->ngrid, na));
  OPAW_CHECK(upload(&c->d_nlm, s->nlm, na));
  OPAW_CHECK(upload(&c->d_goff, c->h_goff.data(), na + 1));
  OPAW_CHECK(upload(&c->d_g3off, c->h_g3off.data(), na + 1));
  OPAW_CHECK(upload(&c->d_qoff, c->h_qoff.data(), na + 1));
  OPAW_CHECK(upload(&c->d_eoff, c->h_eoff.data(), na + 1));
  OPAW_CHECK(upload(&c->d_g3d, s->g3d, c->h_g3off[na]));
  OPAW_CHECK(upload(&c->d_qijlm, s->qijlm, c->h_qoff[na]));
  OPAW_CHECK(upload(&c->d_dij0, s->dij0, c->nd));
  OPAW_CHECK(upload(&c->d_eijkl, s->eijkl, c->h_eoff[na]));

  // kinetic tables (ek.f90:18-40)
  const double dd[3] = {c->dx, c->dy, c->dz};
  for (int k = 0; k < 3; k++) {
    std::vector<double> t(nd3[k]);
    std::vector<float> tf(nd3[k]);
    for (int i = 0; i < nd3[k]; i++) {
      const double kk = kcomp(i, nd3[k], dd[k]);
      t[i] = kk * kk;
      tf[i] = (float)t[i];
    }
    OPAW_CHECK(upload(&c->d_k2[k], t.data(), nd3[k]));
    OPAW_CHECK(upload(&c->d_k2f[k], tf.data(), nd3[k]));
  }
  OPAW_CHECK(upload(&c->d_vloc, s->vloc, c->nn));
  OPAW_CHECK(upload(&c->d_ncoret, s->ncoret, c->nn));
  for (int st = 0; st < 2; st++) {
    OPAW_CHECK(upload<double>(&c->d_vks[st], nullptr, c->nn));
    OPAW_CHECK(upload<float>(&c->d_vks_f[st], nullptr, c->nn));
    OPAW_CHECK(upload<double>(&c->d_dij[st], nullptr, c->nd));
    OPAW_CHECK(upload<double>(&c->d_rhoij[st], nullptr, c->nd));
    OPAW_CHECK(upload<double>(&c->d_dens[st], nullptr, c->nn));
    OPAW_CHECK(upload<double>(&c->d_nhat[st], nullptr, c->nn));
    OPAW_CHECK(upload<double>(&c->d_vh[st], nullptr, c->nn));
    OPAW_CHECK(upload<double>(&c->d_vxc[st], nullptr, c->nn));
  }
  OPAW_CHECK(onsite_init(c, s));
  OPAW_CHECK(upload<double>(&c->oxc_dxc, nullptr, c->nd));
  OPAW_CHECK(fft3_init(c->fft, c->nx, c->ny, c->nz));
  OPAW_CHECK(fft3_init(c->fftb, c->nxb, c->nyb, c->nzb));
  OPAW_CUDA(cudaMallocHost(&c->h_red, 4096 * sizeof(double)));
  // the uploads above went through the legacy stream; the context stream is
  // non-blocking, so make them complete before any kernel reads them
  OPAW_CUDA(cudaDeviceSynchronize());
  OPAW_CHECK(vk_prep(c));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return OPAW_OK;
}

static void destroy(opaw_ctx *c) {
  void *ptrs[] = {c->d_ms, c->d_nrough, c->d_ir0, c->d_poff, c->d_soff, c->d_doff, c->d_p3d, c->d_p3d1,
                  c->d_p3d_f, c->d_p3d1_f, c->d_s, c->d_sinv, c->d_slot_atom, c->d_dslot_atom, c->d_upt,
                  c->d_ustart, c->d_uatom, c->d_ubox, c->d_uent, c->d_utile, c->d_utile_na, c->d_ngrid, c->d_nlm, c->d_goff, c->d_g3off, c->d_qoff,
                  c->d_eoff, c->d_gpt, c->d_g3d, c->d_qijlm, c->d_dij0, c->d_eijkl, c->d_cpt, c->d_cstart,
                  c->d_catom, c->d_cig, c->d_vloc, c->d_ncoret, c->d_vk, c->d_vk_f};
  for (void *p : ptrs) cudaFree(p);
  for (int k = 0; k < 4; k++) cudaFree(c->d_sigma[k]);
  for (int k = 0; k < 3; k++) {
    cudaFree(c->d_k2[k]);
    cudaFree(c->d_k2f[k]);
  }
  for (int st = 0; st < 2; st++) {
    void *sp[] = {c->d_vks[st], c->d_vks_f[st], c->d_dij[st], c->d_rhoij[st], c->d_dens[st],
                  c->d_nhat[st], c->d_vh[st], c->d_vxc[st], c->d_psi[st]};
    for (void *p : sp) cudaFree(p);
  }
  cudaFree(c->d_kgamma);
  onsite_free(c);
  cudaFree(c->oxc_dxc);
  tune_free(c);
  for (auto &b : c->work) cudaFree(b.p);
  for (auto &b : c->coef) cudaFree(b.p);
  cudaFree(c->coefr.p);
  cudaFree(c->gram.p);
  cudaFree(c->gramout.p);
  cudaFree(c->d_boxg);
  cudaFree(c->d_boff);
  cudaFree(c->d_uidx);
  cudaFree(c->d_ovl_start);
  cudaFree(c->d_ovl_atom);
  cudaFree(c->d_ovl_off);
  for (int k = 0; k < 4; k++) cudaFree(c->d_ovl[k]);
  for (auto &b : c->mix) cudaFree(b.p);
  for (cudaEvent_t e : c->kev) cudaEventDestroy(e);
  cudaFree(c->red.p);
  cudaFree(c->pre.p);
  cudaFree(c->g2part.p);
  cudaFree(c->g2other.p);
  cudaFree(c->ddsplit.p);
  cudaFree(c->href.p);
  cudaFree(c->d_tma_err);
  if (c->h_red) cudaFreeHost(c->h_red);
  fft3_free(c->fft);
  fft3_free(c->fftb);
  if (c->side) cudaStreamSynchronize(c->side);
  if (c->side_fork) cudaEventDestroy(c->side_fork);
  if (c->side_join) cudaEventDestroy(c->side_join);
  if (c->side) cudaStreamDestroy(c->side);
  cudaFree(c->oxc_sets.p);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

// a device array of n elements of T with room for K kicks: slot 0 keeps the
// old contents, the new slots start at zero
template <typename T> static int grow_kicks(T **p, size_t n, int K) {
  T *q = nullptr;
  OPAW_CUDA(cudaMalloc(&q, sizeof(T) * n * (size_t)K));
  OPAW_CUDA(cudaMemset(q, 0, sizeof(T) * n * (size_t)K));
  if (*p) OPAW_CUDA(cudaMemcpy(q, *p, sizeof(T) * n, cudaMemcpyDeviceToDevice));
  cudaFree(*p);
  *p = q;
  return OPAW_OK;
}

int kick_capacity(opaw_ctx *c, int K) {
  if (K <= c->kcap && c->d_kgamma) return OPAW_OK;
  if (K > c->kcap) {
    OPAW_CUDA(cudaStreamSynchronize(c->stream));
    OPAW_CHECK(grow_kicks(&c->d_vks[1], c->nn, K));
    OPAW_CHECK(grow_kicks(&c->d_vks_f[1], c->nn, K));
    OPAW_CHECK(grow_kicks(&c->d_dij[1], c->nd, K));
    OPAW_CHECK(grow_kicks(&c->d_rhoij[1], c->nd, K));
    OPAW_CHECK(grow_kicks(&c->d_dens[1], c->nn, K));
    OPAW_CHECK(grow_kicks(&c->d_nhat[1], c->nn, K));
    OPAW_CHECK(grow_kicks(&c->d_vh[1], c->nn, K));
    OPAW_CHECK(grow_kicks(&c->d_vxc[1], c->nn, K));
    c->kcap = K;
    cudaFree(c->d_kgamma);
    c->d_kgamma = nullptr;
  }
  OPAW_CUDA(cudaMalloc(&c->d_kgamma, sizeof(double) * (size_t)c->kcap));
  return OPAW_OK;
}

int upload_kgamma(opaw_ctx *c) {
  OPAW_CHECK(kick_capacity(c, c->nkick));
  OPAW_ARG((int)c->h_kgamma.size() >= c->nkick, "kick strengths missing");
  OPAW_CUDA(cudaMemcpyAsync(c->d_kgamma, c->h_kgamma.data(), sizeof(double) * c->nkick, cudaMemcpyHostToDevice,
                            c->stream));
  return OPAW_OK;
}

// float twin of v_ks for the mixed-precision operators
__global__ void k_to_float(const double *__restrict__ a, float *__restrict__ b, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

int refresh_vks_f(opaw_ctx *c, int set) {
  k_to_float<<<grid1(c->nn, 256), 256, 0, c->stream>>>(c->d_vks[set], c->d_vks_f[set], c->nn);
  c->launches++;
  OPAW_CUDA(cudaGetLastError());
  return OPAW_OK;
}

static int check_ctx(opaw_ctx *c) {
  if (!c) {
    set_error("null context");
    return OPAW_ERR_ARG;
  }
  return OPAW_OK;
}
static int check_set(int set) {
  if (set != 0 && set != 1) {
    set_error("set must be 0 (unperturbed) or 1 (perturbed)");
    return OPAW_ERR_ARG;
  }
  return OPAW_OK;
}

}  // namespace opaw

using namespace opaw;

extern "C" {

const char *opaw_last_error(void) { return get_error(); }

int opaw_dev_init(const opaw_system *sys, opaw_ctx **out) {
  if (!sys || !out) {
    set_error("null argument");
    return OPAW_ERR_ARG;
  }
  *out = nullptr;
  if (sys->nx <= 0 || sys->ny <= 0 || sys->nz <= 0 || !(sys->dx > 0) || !(sys->dy > 0) || !(sys->dz > 0) ||
      sys->natom < 0) {
    set_error("grid extents and spacings must be positive");
    return OPAW_ERR_ARG;
  }
  if (sys->natom > 0 && (!sys->ir_start || !sys->nrough || !sys->ms || !sys->p3d || !sys->p3d1 || !sys->s ||
                         !sys->sinv || !sys->ngrid || !sys->nlm || !sys->dij0 || !sys->eijkl)) {
    set_error("atom tables missing");
    return OPAW_ERR_ARG;
  }
  if (!sys->vloc || !sys->ncoret) {
    set_error("vloc and ncoret are required");
    return OPAW_ERR_ARG;
  }
  {
    // host-side validation of the tables before touching a device
    const int nd3[3] = {sys->nx, sys->ny, sys->nz};
    int64_t ng = 0;
    for (int a = 0; a < sys->natom; a++) {
      if (sys->ms[a] < 1 || sys->ms[a] > 16) {
        set_error("projectors per atom must be in [1, 16]");
        return OPAW_ERR_ARG;
      }
      for (int k = 0; k < 3; k++) {
        const int nr = sys->nrough[3 * a + k], i0 = sys->ir_start[3 * a + k] - 1;
        if (nr <= 0 || nr > nd3[k]) {
          set_error("projector box larger than the grid (read_paw.f90:254)");
          return OPAW_ERR_ARG;
        }
        if (!sys->periodic && (i0 < 0 || i0 + nr > nd3[k])) {
          set_error("non periodic, local grid cannot go outside box: atom " + std::to_string(a + 1));
          return OPAW_ERR_BOX;  // get_irs.f90:30-35
        }
        if (i0 <= -nd3[k] || i0 >= nd3[k]) {
          set_error("box origin more than one period outside the grid");
          return OPAW_ERR_ARG;
        }
      }
      if (sys->ngrid[a] < 0 || sys->nlm[a] < 0 || sys->nlm[a] > 64) {
        set_error("bad compensation-sphere sizes");
        return OPAW_ERR_ARG;
      }
      ng += sys->ngrid[a];
    }
    if (ng > 0 && !sys->local_grid) {
      set_error("local_grid missing");
      return OPAW_ERR_ARG;
    }
    for (int64_t i = 0; i < 3 * ng; i++) {
      const int v = sys->local_grid[i];
      if (v < 1 || v > nd3[i % 3]) {
        set_error("compensation-sphere point outside the grid");
        return OPAW_ERR_ARG;
      }
    }
    for (int k = 0; k < 3; k++) {
      int m = nd3[k];
      for (int r : {2, 3, 5, 7, 11, 13})
        while (m % r == 0) m /= r;
      if (m != 1) {
        set_error("grid extent " + std::to_string(nd3[k]) + " has a prime factor other than 2, 3, 5, 7, 11, 13");
        return OPAW_ERR_ARG;
      }
    }
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("no CUDA device");
    return OPAW_ERR_NODEV;
  }
  opaw_ctx *c = new opaw_ctx();
  int st = build(c, sys);
  if (st != OPAW_OK) {
    std::string keep = get_error();
    destroy(c);
    set_error(keep);
    return st;
  }
  *out = c;
  return OPAW_OK;
}

int opaw_dev_free(opaw_ctx *c) {
  if (!c) return OPAW_OK;
  cudaStreamSynchronize(c->stream);
  destroy(c);
  return OPAW_OK;
}

void *opaw_stream(opaw_ctx *c) { return c ? (void *)c->stream : nullptr; }
int64_t opaw_kernel_launches(opaw_ctx *c) { return c ? c->launches : 0; }

int opaw_ktime_begin(opaw_ctx *c) {
  OPAW_CHECK(check_ctx(c));
  c->ktime_on = true;
  c->kev_used = 0;
  c->kbytes = 0.0;
  return OPAW_OK;
}

int opaw_ktime_end(opaw_ctx *c, double *ms, int *launches, double *bytes) {
  OPAW_CHECK(check_ctx(c));
  c->ktime_on = false;
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  double tot = 0.0;
  for (int i = 0; i + 1 < c->kev_used; i += 2) {
    float t = 0.f;
    OPAW_CUDA(cudaEventElapsedTime(&t, c->kev[i], c->kev[i + 1]));
    tot += t;
  }
  if (ms) *ms = tot;
  if (launches) *launches = c->kev_used / 2;
  if (bytes) *bytes = c->kbytes;
  return OPAW_OK;
}

int opaw_sync(opaw_ctx *c) {
  OPAW_CHECK(check_ctx(c));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return tma_status(c);
}

int opaw_psi_upload(opaw_ctx *c, int set, const double *psi, int norb) {
  OPAW_CHECK(check_ctx(c));
  OPAW_CHECK(check_set(set));
  OPAW_ARG(psi && norb > 0, "psi must be non-null with norb > 0");
  if (c->norb[set] != norb || (set == 1 && c->nkick != 1)) {
    OPAW_CUDA(cudaStreamSynchronize(c->stream));
    cudaFree(c->d_psi[set]);
    c->d_psi[set] = nullptr;
    OPAW_CUDA(cudaMalloc(&c->d_psi[set], sizeof(double2) * (size_t)c->nn * norb));
    c->norb[set] = norb;
  }
  if (set == 1) c->nkick = 1;  // one kicked set, uploaded as it is
  if (set == 0) c->psi0_gen++;
  OPAW_CUDA(cudaMemcpyAsync(c->d_psi[set], psi, sizeof(double2) * (size_t)c->nn * norb, cudaMemcpyHostToDevice,
                            c->stream));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return OPAW_OK;
}

int opaw_psi_download(opaw_ctx *c, int set, double *psi, int norb) {
  OPAW_CHECK(check_ctx(c));
  OPAW_CHECK(check_set(set));
  OPAW_ARG(psi, "psi must be non-null");
  if (c->norb[set] == 0) {
    set_error("no orbitals uploaded for this set");
    return OPAW_ERR_STATE;
  }
  OPAW_ARG(norb == c->norb[set], "norb differs from the uploaded count");
  OPAW_CUDA(cudaMemcpyAsync(psi, c->d_psi[set], sizeof(double2) * (size_t)c->nn * norb, cudaMemcpyDeviceToHost,
                            c->stream));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return OPAW_OK;
}

void *opaw_psi_device(opaw_ctx *c, int set) {
  if (!c || (set != 0 && set != 1)) return nullptr;
  if (set == 0) c->psi0_gen++;  // the caller may write through the pointer
  return c->d_psi[set];
}

static int put(opaw_ctx *c, void *dst, const void *src, size_t bytes) {
  OPAW_ARG(src, "null input");
  OPAW_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return OPAW_OK;
}
static int get(opaw_ctx *c, void *dst, const void *src, size_t bytes) {
  OPAW_ARG(dst, "null output");
  OPAW_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->stream));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return OPAW_OK;
}

int opaw_set_vks(opaw_ctx *c, int set, const double *vks) {
  OPAW_CHECK(check_ctx(c));
  OPAW_CHECK(check_set(set));
  OPAW_CHECK(put(c, c->d_vks[set], vks, sizeof(double) * c->nn));
  OPAW_CHECK(refresh_vks_f(c, set));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return OPAW_OK;
}
int opaw_get_vks(opaw_ctx *c, int set, double *v) {
  OPAW_CHECK(check_ctx(c)); OPAW_CHECK(check_set(set));
  return get(c, v, c->d_vks[set], sizeof(double) * c->nn);
}
int opaw_set_dij(opaw_ctx *c, int set, const double *d) {
  OPAW_CHECK(check_ctx(c)); OPAW_CHECK(check_set(set));
  return put(c, c->d_dij[set], d, sizeof(double) * c->nd);
}
int opaw_get_dij(opaw_ctx *c, int set, double *d) {
  OPAW_CHECK(check_ctx(c)); OPAW_CHECK(check_set(set));
  return get(c, d, c->d_dij[set], sizeof(double) * c->nd);
}
int opaw_get_rhoij(opaw_ctx *c, int set, double *d) {
  OPAW_CHECK(check_ctx(c)); OPAW_CHECK(check_set(set));
  return get(c, d, c->d_rhoij[set], sizeof(double) * c->nd);
}
int opaw_get_density(opaw_ctx *c, int set, double *d) {
  OPAW_CHECK(check_ctx(c)); OPAW_CHECK(check_set(set));
  return get(c, d, c->d_dens[set], sizeof(double) * c->nn);
}
int opaw_get_nhat(opaw_ctx *c, int set, double *d) {
  OPAW_CHECK(check_ctx(c)); OPAW_CHECK(check_set(set));
  return get(c, d, c->d_nhat[set], sizeof(double) * c->nn);
}

// ---- per-routine operators over device buffers (asynchronous on the stream)

int opaw_h_apply_dev(opaw_ctx *c, int set, int dtype, const void *pin, void *hp, int norb) {
  OPAW_CHECK(check_ctx(c)); OPAW_CHECK(check_set(set));
  OPAW_ARG(pin && hp && norb >= 0, "bad buffers");
  if (dtype == OPAW_C128) return h_apply<double>(c, set, (const double2 *)pin, (double2 *)hp, norb);
  if (dtype == OPAW_C64) return h_apply<float>(c, set, (const float2 *)pin, (float2 *)hp, norb);
  set_error("dtype must be OPAW_C128 or OPAW_C64");
  return OPAW_ERR_ARG;
}

int opaw_precond_kinetic_dev(opaw_ctx *c, int dtype, const void *pin, const double *ekin, void *out, int norb) {
  OPAW_CHECK(check_ctx(c));
  OPAW_ARG(pin && out && ekin && norb >= 0, "bad buffers");
  if (norb == 0) return OPAW_OK;
  std::vector<double> inv(norb);
  for (int i = 0; i < norb; i++) {
    OPAW_ARG(ekin[i] > 0.0 && std::isfinite(ekin[i]), "kinetic energies must be positive and finite");
    inv[i] = 1.0 / ekin[i];
  }
  OPAW_CHECK(ensure(c->pre, sizeof(double) * (size_t)norb));
  OPAW_CUDA(cudaMemcpyAsync(c->pre.p, inv.data(), sizeof(double) * norb, cudaMemcpyHostToDevice, c->stream));
  if (dtype == OPAW_C128)
    return precond_kinetic<double>(c, (const double2 *)pin, (const double *)c->pre.p, (double2 *)out, norb);
  if (dtype == OPAW_C64)
    return precond_kinetic<float>(c, (const float2 *)pin, (const double *)c->pre.p, (float2 *)out, norb);
  set_error("dtype must be OPAW_C128 or OPAW_C64");
  return OPAW_ERR_ARG;
}

int opaw_kinetic_energy_dev(opaw_ctx *c, int dtype, const void *x, int norb, double *ekin) {
  OPAW_CHECK(check_ctx(c));
  OPAW_ARG(x && ekin && norb >= 0, "bad buffers");
  if (dtype == OPAW_C128) return kinetic_energy<double>(c, (const double2 *)x, norb, ekin);
  if (dtype == OPAW_C64) return kinetic_energy<float>(c, (const float2 *)x, norb, ekin);
  set_error("dtype must be OPAW_C128 or OPAW_C64");
  return OPAW_ERR_ARG;
}

int opaw_sn_apply_dev(opaw_ctx *c, int dtype, double n, const void *pin, void *sp, int norb) {
  OPAW_CHECK(check_ctx(c));
  OPAW_ARG(pin && sp && norb >= 0, "bad buffers");
  if (dtype == OPAW_C128) return sn_apply<double>(c, n, (const double2 *)pin, (double2 *)sp, norb);
  if (dtype == OPAW_C64) return sn_apply<float>(c, n, (const float2 *)pin, (float2 *)sp, norb);
  set_error("dtype must be OPAW_C128 or OPAW_C64");
  return OPAW_ERR_ARG;
}

int opaw_shs_apply_dev(opaw_ctx *c, int set, int dtype, const void *pin, void *pout, int norb) {
  OPAW_CHECK(check_ctx(c)); OPAW_CHECK(check_set(set));
  OPAW_ARG(pin && pout && norb >= 0, "bad buffers");
  OPAW_ARG(pin != pout, "shs needs distinct input and output buffers");
  if (dtype == OPAW_C128) return shs_apply<double>(c, set, (const double2 *)pin, (double2 *)pout, norb);
  if (dtype == OPAW_C64) return shs_apply<float>(c, set, (const float2 *)pin, (float2 *)pout, norb);
  set_error("dtype must be OPAW_C128 or OPAW_C64");
  return OPAW_ERR_ARG;
}

int opaw_proj_dev(opaw_ctx *c, int which, int dtype, const void *pin, int norb, double *ca) {
  OPAW_CHECK(check_ctx(c));
  OPAW_ARG(pin && ca && norb > 0 && (which == 0 || which == 1), "bad arguments");
  OPAW_CHECK(ensure(c->coef[0], sizeof(double2) * (size_t)c->ns * norb + 16));
  double2 *co = (double2 *)c->coef[0].p;
  if (dtype == OPAW_C128) OPAW_CHECK(gather<double>(c, which, (const double2 *)pin, norb, co));
  else if (dtype == OPAW_C64) OPAW_CHECK(gather<float>(c, which, (const float2 *)pin, norb, co));
  else {
    set_error("dtype must be OPAW_C128 or OPAW_C64");
    return OPAW_ERR_ARG;
  }
  return get(c, ca, co, sizeof(double2) * (size_t)c->ns * norb);
}

int opaw_fft3d_dev(opaw_ctx *c, int dtype, void *data, int norb, int sign) {
  OPAW_CHECK(check_ctx(c));
  OPAW_ARG(data && norb >= 0 && (sign == -1 || sign == 1), "bad arguments");
  if (norb == 0) return OPAW_OK;
  if (dtype == OPAW_C128) return fft3d<double>(c, c->fft, (double2 *)data, norb, sign);
  if (dtype == OPAW_C64) return fft3d<float>(c, c->fft, (float2 *)data, norb, sign);
  set_error("dtype must be OPAW_C128 or OPAW_C64");
  return OPAW_ERR_ARG;
}

// ---- host-buffer twins: copy in, apply in the requested precision, copy out

__global__ void k_c128_to_c64(const double2 *__restrict__ a, float2 *__restrict__ b, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = make_float2((float)a[i].x, (float)a[i].y);
}
__global__ void k_c64_to_c128(const float2 *__restrict__ a, double2 *__restrict__ b, int64_t n) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = make_double2((double)a[i].x, (double)a[i].y);
}

static int host_op(opaw_ctx *c, int kind, int set, int dtype, double n, const double *pin, double *out, int norb) {
  OPAW_CHECK(check_ctx(c));
  OPAW_ARG(pin && out && norb > 0, "bad buffers");
  const int64_t tot = c->nn * (int64_t)norb;
  OPAW_CHECK(ensure(c->work[5], sizeof(double2) * tot));
  OPAW_CHECK(ensure(c->work[6], sizeof(double2) * tot));
  double2 *a = (double2 *)c->work[5].p, *b = (double2 *)c->work[6].p;
  OPAW_CUDA(cudaMemcpyAsync(a, pin, sizeof(double2) * tot, cudaMemcpyHostToDevice, c->stream));
  if (dtype == OPAW_C128) {
    if (kind == 0) OPAW_CHECK(h_apply<double>(c, set, a, b, norb));
    else if (kind == 1) OPAW_CHECK(sn_apply<double>(c, n, a, b, norb));
    else OPAW_CHECK(shs_apply<double>(c, set, a, b, norb));
  } else if (dtype == OPAW_C64) {
    float2 *af = (float2 *)b, *bf = (float2 *)a;  // c64 views: a -> b(f32) -> a(f32)
    k_c128_to_c64<<<grid1(tot, 256), 256, 0, c->stream>>>(a, af, tot);
    c->launches++;
    if (kind == 0) OPAW_CHECK(h_apply<float>(c, set, af, bf, norb));
    else if (kind == 1) OPAW_CHECK(sn_apply<float>(c, n, af, bf, norb));
    else OPAW_CHECK(shs_apply<float>(c, set, af, bf, norb));
    k_c64_to_c128<<<grid1(tot, 256), 256, 0, c->stream>>>(bf, b, tot);
    c->launches++;
  } else {
    set_error("dtype must be OPAW_C128 or OPAW_C64");
    return OPAW_ERR_ARG;
  }
  OPAW_CUDA(cudaGetLastError());
  OPAW_CUDA(cudaMemcpyAsync(out, b, sizeof(double2) * tot, cudaMemcpyDeviceToHost, c->stream));
  OPAW_CUDA(cudaStreamSynchronize(c->stream));
  return OPAW_OK;
}

int opaw_h_phi(opaw_ctx *c, int set, int dtype, const double *pin, double *hp, int norb) {
  OPAW_CHECK(check_set(set));
  return host_op(c, 0, set, dtype, 0.0, pin, hp, norb);
}
int opaw_sn_phi(opaw_ctx *c, int dtype, double n, const double *pin, double *sp, int norb) {
  return host_op(c, 1, 0, dtype, n, pin, sp, norb);
}
int opaw_shs(opaw_ctx *c, int set, int dtype, const double *pin, double *pout, int norb) {
  OPAW_CHECK(check_set(set));
  return host_op(c, 2, set, dtype, 0.0, pin, pout, norb);
}

}  // extern "C"
