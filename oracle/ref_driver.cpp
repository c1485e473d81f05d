// ref_driver.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Loop driver around the reference's own pair and panel kernels.  This file is not
// compiled on its own: oracle/build_ref.sh streams the reference's MathHelper.h,
// CoreFunc.h (with the core selection line switched) and Kernels.h into the compiler
// ahead of it, so every call below lands in the reference's arithmetic.  The loops are
// restated from the reference's non-Vc x86 branches (the files that hold them need
// Eigen/Vc and cannot be built here):
//   points_affect_points   Influence.h:278-309, :312-366, :445-475, :477-534
//   panels_affect_points   Influence.h:948-1000 (and its velocity-only sibling)
//   points_affect_panels   Influence.h:1192-1215
//   panels_on_panels_coeff Coefficients.h:334-447
// Outputs are written into oracle/_ref/libo3dref_<core>.so and are used only to pin
// the oracle restatement (oracle/o3d_oracle.cpp) and to generate tests/golden/.

#include <cstdint>
#include <cstddef>
#include <cmath>

#ifndef RECURSIVE_LEVELS_REF
#define RECURSIVE_LEVELS_REF 3
#endif

namespace {

template <class S, class A>
void ref_ptpt(int ns, const S* sx, const S* sr, const S* ss, int nt, const S* tx, const S* tr, S* tu, S* tug) {
  const S* sy = sx + ns; const S* sz = sx + 2 * (size_t)ns;
  const S* ssx = ss; const S* ssy = ss + ns; const S* ssz = ss + 2 * (size_t)ns;
  const S* ty = tx + nt; const S* tz = tx + 2 * (size_t)nt;
  S* tv = tu + nt; S* tw = tu + 2 * (size_t)nt;
  #pragma omp parallel for
  for (int32_t i = 0; i < nt; ++i) {
    if (tug) {
      A accumu = 0.0, accumv = 0.0, accumw = 0.0;
      A accumux = 0.0, accumvx = 0.0, accumwx = 0.0;
      A accumuy = 0.0, accumvy = 0.0, accumwy = 0.0;
      A accumuz = 0.0, accumvz = 0.0, accumwz = 0.0;
      if (tr) {
        for (size_t j = 0; j < (size_t)ns; ++j)
          kernel_0v_0bg<S, A>(sx[j], sy[j], sz[j], sr[j], ssx[j], ssy[j], ssz[j], tx[i], ty[i], tz[i], tr[i],
                              &accumu, &accumv, &accumw, &accumux, &accumvx, &accumwx,
                              &accumuy, &accumvy, &accumwy, &accumuz, &accumvz, &accumwz);
      } else {
        for (size_t j = 0; j < (size_t)ns; ++j)
          kernel_0v_0pg<S, A>(sx[j], sy[j], sz[j], sr[j], ssx[j], ssy[j], ssz[j], tx[i], ty[i], tz[i],
                              &accumu, &accumv, &accumw, &accumux, &accumvx, &accumwx,
                              &accumuy, &accumvy, &accumwy, &accumuz, &accumvz, &accumwz);
      }
      tu[i] += accumu; tv[i] += accumv; tw[i] += accumw;
      const A g[9] = {accumux, accumvx, accumwx, accumuy, accumvy, accumwy, accumuz, accumvz, accumwz};
      for (int d = 0; d < 9; ++d) tug[d * (size_t)nt + i] += g[d];
    } else {
      A accumu = 0.0, accumv = 0.0, accumw = 0.0;
      if (tr) {
        for (size_t j = 0; j < (size_t)ns; ++j)
          kernel_0v_0b<S, A>(sx[j], sy[j], sz[j], sr[j], ssx[j], ssy[j], ssz[j], tx[i], ty[i], tz[i], tr[i],
                             &accumu, &accumv, &accumw);
      } else {
        for (size_t j = 0; j < (size_t)ns; ++j)
          kernel_0v_0p<S, A>(sx[j], sy[j], sz[j], sr[j], ssx[j], ssy[j], ssz[j], tx[i], ty[i], tz[i],
                             &accumu, &accumv, &accumw);
      }
      tu[i] += accumu; tv[i] += accumv; tw[i] += accumw;
    }
  }
}

template <class S, class A>
void ref_panpt(int maxlev, int nn, const S* nx, int np, const uint32_t* si, const S* sa, const S* ts,
               const S* sss, int nt, const S* tx, S* tu, S* tug) {
  const S* ny = nx + nn; const S* nz = nx + 2 * (size_t)nn;
  const S* ty = tx + nt; const S* tz = tx + 2 * (size_t)nt;
  #pragma omp parallel for schedule(dynamic, 16)
  for (int32_t i = 0; i < nt; ++i) {
    A accumu = 0.0, accumv = 0.0, accumw = 0.0;
    A accumux = 0.0, accumvx = 0.0, accumwx = 0.0;
    A accumuy = 0.0, accumvy = 0.0, accumwy = 0.0;
    A accumuz = 0.0, accumvz = 0.0, accumwz = 0.0;
    for (size_t j = 0; j < (size_t)np; ++j) {
      const size_t jp0 = si[3 * j], jp1 = si[3 * j + 1], jp2 = si[3 * j + 2];
      const S srcs = sss ? sss[j] : S(0.0);
      if (tug) {
        rkernel_2vs_0pg<S, A>(nx[jp0], ny[jp0], nz[jp0], nx[jp1], ny[jp1], nz[jp1], nx[jp2], ny[jp2], nz[jp2],
                              ts[j] / sa[j], ts[np + j] / sa[j], ts[2 * (size_t)np + j] / sa[j], srcs,
                              tx[i], ty[i], tz[i], sa[j], 0, maxlev,
                              &accumu, &accumv, &accumw, &accumux, &accumvx, &accumwx,
                              &accumuy, &accumvy, &accumwy, &accumuz, &accumvz, &accumwz);
      } else {
        rkernel_2vs_0p<S, A>(nx[jp0], ny[jp0], nz[jp0], nx[jp1], ny[jp1], nz[jp1], nx[jp2], ny[jp2], nz[jp2],
                             ts[j] / sa[j], ts[np + j] / sa[j], ts[2 * (size_t)np + j] / sa[j], srcs,
                             tx[i], ty[i], tz[i], sa[j], 0, maxlev, &accumu, &accumv, &accumw);
      }
    }
    tu[i] += accumu; tu[nt + (size_t)i] += accumv; tu[2 * (size_t)nt + i] += accumw;
    if (tug) {
      const A g[9] = {accumux, accumvx, accumwx, accumuy, accumvy, accumwy, accumuz, accumvz, accumwz};
      for (int d = 0; d < 9; ++d) tug[d * (size_t)nt + i] += g[d];
    }
  }
}

template <class S, class A>
void ref_ptpan(int maxlev, int ns, const S* sx, const S* ss, int nn, const S* nx, int np, const uint32_t* ti,
               const S* ta, S* pu) {
  const S* sy = sx + ns; const S* sz = sx + 2 * (size_t)ns;
  const S* ny = nx + nn; const S* nz = nx + 2 * (size_t)nn;
  #pragma omp parallel for schedule(dynamic, 4)
  for (int32_t i = 0; i < np; ++i) {
    A accumu = 0.0, accumv = 0.0, accumw = 0.0;
    const size_t ip0 = ti[3 * (size_t)i], ip1 = ti[3 * (size_t)i + 1], ip2 = ti[3 * (size_t)i + 2];
    for (size_t j = 0; j < (size_t)ns; ++j) {
      rkernel_2vs_0p<S, A>(nx[ip0], ny[ip0], nz[ip0], nx[ip1], ny[ip1], nz[ip1], nx[ip2], ny[ip2], nz[ip2],
                           ss[j] / ta[i], ss[ns + j] / ta[i], ss[2 * (size_t)ns + j] / ta[i], S(0.0),
                           sx[j], sy[j], sz[j], ta[i], 0, maxlev, &accumu, &accumv, &accumw);
    }
    pu[i] -= accumu; pu[np + (size_t)i] -= accumv; pu[2 * (size_t)np + i] -= accumw;
  }
}

template <class S>
void ref_coeff(int maxlev, int nunk, int is_self, int snn, const S* sxx, int nsrc, const uint32_t* si, const S* sa,
               const S* sb1, const S* sb2, int tnn, const S* txx, int ntarg, const uint32_t* ti, const S* ta,
               const S* tb1, const S* tb2, const S* tn, S* coeffs) {
  const bool targ_has_src = (nunk == 3), src_has_src = (nunk == 3);
  const size_t snunk = nunk, tnunk = nunk;
  const S* sxy = sxx + snn; const S* sxz = sxx + 2 * (size_t)snn;
  const S* txy = txx + tnn; const S* txz = txx + 2 * (size_t)tnn;
  #pragma omp parallel for schedule(dynamic, 4)
  for (int32_t j = 0; j < nsrc; j++) {
    size_t jptr[3];
    for (size_t i = 0; i < snunk; ++i) jptr[i] = (j * snunk + i) * (ntarg * tnunk);
    const uint32_t sfirst = si[3 * (size_t)j], ssecond = si[3 * (size_t)j + 1], sthird = si[3 * (size_t)j + 2];
    const S sx0 = sxx[sfirst], sy0 = sxy[sfirst], sz0 = sxz[sfirst];
    const S sx1 = sxx[ssecond], sy1 = sxy[ssecond], sz1 = sxz[ssecond];
    const S sx2 = sxx[sthird], sy2 = sxy[sthird], sz2 = sxz[sthird];
    const S sarea = sa[j];
    for (size_t i = 0; i < (size_t)ntarg; i++) {
      const uint32_t tfirst = ti[3 * i], tsecond = ti[3 * i + 1], tthird = ti[3 * i + 2];
      for (size_t k = 0; k < snunk; ++k) {
        S resultu = 0.0, resultv = 0.0, resultw = 0.0;
        if (k == 0)
          rkernel_2vs_2p<S, S>(sx0, sy0, sz0, sx1, sy1, sz1, sx2, sy2, sz2,
                               sb1[j], sb1[nsrc + j], sb1[2 * (size_t)nsrc + j], S(0.0),
                               txx[tfirst], txy[tfirst], txz[tfirst], txx[tsecond], txy[tsecond], txz[tsecond],
                               txx[tthird], txy[tthird], txz[tthird], sarea, ta[i], 0, maxlev,
                               &resultu, &resultv, &resultw);
        else if (k == 1)
          rkernel_2vs_2p<S, S>(sx0, sy0, sz0, sx1, sy1, sz1, sx2, sy2, sz2,
                               sb2[j], sb2[nsrc + j], sb2[2 * (size_t)nsrc + j], S(0.0),
                               txx[tfirst], txy[tfirst], txz[tfirst], txx[tsecond], txy[tsecond], txz[tsecond],
                               txx[tthird], txy[tthird], txz[tthird], sarea, ta[i], 0, maxlev,
                               &resultu, &resultv, &resultw);
        else
          rkernel_2vs_2p<S, S>(sx0, sy0, sz0, sx1, sy1, sz1, sx2, sy2, sz2,
                               (S)0.0, (S)0.0, (S)0.0, (S)1.0,
                               txx[tfirst], txy[tfirst], txz[tfirst], txx[tsecond], txy[tsecond], txz[tsecond],
                               txx[tthird], txy[tthird], txz[tthird], sarea, ta[i], 0, maxlev,
                               &resultu, &resultv, &resultw);
        if (k == 2 && !src_has_src) continue;
        coeffs[jptr[k]++] = resultu * tb1[i] + resultv * tb1[ntarg + i] + resultw * tb1[2 * (size_t)ntarg + i];
        coeffs[jptr[k]++] = resultu * tb2[i] + resultv * tb2[ntarg + i] + resultw * tb2[2 * (size_t)ntarg + i];
        if (targ_has_src)
          coeffs[jptr[k]++] = resultu * tn[i] + resultv * tn[ntarg + i] + resultw * tn[2 * (size_t)ntarg + i];
      }
    }
    if (is_self) {
      size_t dptr = j * ntarg * nunk * nunk + j * nunk;
      coeffs[dptr] = 0.0;
      coeffs[dptr + 1] = 2.0 * M_PI;
      if (targ_has_src) coeffs[dptr + 2] = 0.0;
      dptr += ntarg * nunk;
      coeffs[dptr] = -2.0 * M_PI;
      coeffs[dptr + 1] = 0.0;
      if (targ_has_src) coeffs[dptr + 2] = 0.0;
      if (src_has_src) {
        dptr += ntarg * nunk;
        coeffs[dptr] = 0.0;
        coeffs[dptr + 1] = 0.0;
        if (targ_has_src) coeffs[dptr + 2] = 2.0 * M_PI;
      }
    }
  }
  const S fac = 1.0 / (4.0 * M_PI);
  const size_t ntot = (size_t)ntarg * tnunk * (size_t)nsrc * snunk;
  for (size_t e = 0; e < ntot; ++e) coeffs[e] = coeffs[e] * fac;
}

}  // namespace

extern "C" {

int ref_points_affect_points(int prec, int ns, const void* sx, const void* sr, const void* ss, int nt,
                             const void* tx, const void* tr, void* tu, void* tug) {
  if (prec == 0)
    ref_ptpt<float, float>(ns, (const float*)sx, (const float*)sr, (const float*)ss, nt, (const float*)tx,
                           (const float*)tr, (float*)tu, (float*)tug);
  else if (prec == 1)
    ref_ptpt<float, double>(ns, (const float*)sx, (const float*)sr, (const float*)ss, nt, (const float*)tx,
                            (const float*)tr, (float*)tu, (float*)tug);
  else if (prec == 2)
    ref_ptpt<double, double>(ns, (const double*)sx, (const double*)sr, (const double*)ss, nt, (const double*)tx,
                             (const double*)tr, (double*)tu, (double*)tug);
  else
    return 1;
  return 0;
}

int ref_panels_affect_points(int prec, int maxlev, int nn, const void* nx, int np, const uint32_t* idx,
                             const void* area, const void* ts, const void* sss, int nt, const void* tx,
                             void* tu, void* tug) {
  if (prec == 0)
    ref_panpt<float, float>(maxlev, nn, (const float*)nx, np, idx, (const float*)area, (const float*)ts,
                            (const float*)sss, nt, (const float*)tx, (float*)tu, (float*)tug);
  else if (prec == 1)
    ref_panpt<float, double>(maxlev, nn, (const float*)nx, np, idx, (const float*)area, (const float*)ts,
                             (const float*)sss, nt, (const float*)tx, (float*)tu, (float*)tug);
  else if (prec == 2)
    ref_panpt<double, double>(maxlev, nn, (const double*)nx, np, idx, (const double*)area, (const double*)ts,
                              (const double*)sss, nt, (const double*)tx, (double*)tu, (double*)tug);
  else
    return 1;
  return 0;
}

int ref_points_affect_panels(int prec, int maxlev, int ns, const void* sx, const void* ss, int nn, const void* nx,
                             int np, const uint32_t* idx, const void* area, void* pu) {
  if (prec == 0)
    ref_ptpan<float, float>(maxlev, ns, (const float*)sx, (const float*)ss, nn, (const float*)nx, np, idx,
                            (const float*)area, (float*)pu);
  else if (prec == 1)
    ref_ptpan<float, double>(maxlev, ns, (const float*)sx, (const float*)ss, nn, (const float*)nx, np, idx,
                             (const float*)area, (float*)pu);
  else if (prec == 2)
    ref_ptpan<double, double>(maxlev, ns, (const double*)sx, (const double*)ss, nn, (const double*)nx, np, idx,
                              (const double*)area, (double*)pu);
  else
    return 1;
  return 0;
}

int ref_panels_on_panels_coeff(int prec, int maxlev, int nunk, int is_self,
                               int snn, const void* snx, int snp, const uint32_t* sidx, const void* sarea,
                               const void* sx1, const void* sx2,
                               int tnn, const void* tnx, int tnp, const uint32_t* tidx, const void* tarea,
                               const void* tx1, const void* tx2, const void* tnorm, void* coeffs) {
  if (prec == 0)
    ref_coeff<float>(maxlev, nunk, is_self, snn, (const float*)snx, snp, sidx, (const float*)sarea,
                     (const float*)sx1, (const float*)sx2, tnn, (const float*)tnx, tnp, tidx, (const float*)tarea,
                     (const float*)tx1, (const float*)tx2, (const float*)tnorm, (float*)coeffs);
  else if (prec == 2)
    ref_coeff<double>(maxlev, nunk, is_self, snn, (const double*)snx, snp, sidx, (const double*)sarea,
                      (const double*)sx1, (const double*)sx2, tnn, (const double*)tnx, tnp, tidx, (const double*)tarea,
                      (const double*)tx1, (const double*)tx2, (const double*)tnorm, (double*)coeffs);
  else
    return 1;
  return 0;
}

}  // extern "C"
