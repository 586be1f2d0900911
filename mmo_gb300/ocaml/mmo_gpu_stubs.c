/*
 * mmo_gpu_stubs.c -- OCaml C stubs over libmmo_gpu.so (include/mmo_gpu.h).
 *
 * The binding a maintainer adds to UnixJunkie/MMO so that the scoring
 * closures of src/lds.ml (ene_inter, src/lds.ml:1952-1979; ene_intra,
 * src/lds.ml:702-712) and Optim's config scoring (src/optim.ml:64-80) run on
 * the GPU.  OCaml float arrays are flat, so their data is passed to the
 * library without a copy; int arrays are converted to C ints.  A non-zero
 * status raises Failure with the library's message; a pose that is too
 * elongated raises the exception registered as "Mol.Too_long" (see
 * ff_gpu.ml), like Optim.apply_config does (src/optim.ml:75).
 *
 * The context is created lazily by the OCaml side, after parany has forked
 * its workers (src/lds.ml:2009,2050): a CUDA context must not cross a fork.
 */
#define CAML_NAME_SPACE
#include <caml/alloc.h>
#include <caml/callback.h>
#include <caml/custom.h>
#include <caml/fail.h>
#include <caml/memory.h>
#include <caml/mlvalues.h>
#include <stdint.h>
#include <stdlib.h>

#include "mmo_grid.h"

#define Ctx_val(v) (*((mmo_ctx **)Data_custom_val(v)))
#define Doubles(v) ((double *)(v))

static void ctx_finalize(value v) {
  mmo_ctx *c = Ctx_val(v);
  if (c) mmo_ctx_destroy(c);
  Ctx_val(v) = NULL;
}

static struct custom_operations ctx_ops = {
    "mmo.gpu.ctx",          ctx_finalize,           custom_compare_default,
    custom_hash_default,    custom_serialize_default, custom_deserialize_default,
    custom_compare_ext_default, custom_fixed_length_default};

static void check(mmo_ctx *c, int rc) {
  if (rc != MMO_OK) caml_failwith(mmo_last_error(c));
}

static int *c_ints(value a) {
  mlsize_t n = Wosize_val(a), i;
  int *p = (int *)malloc(sizeof(int) * (n ? n : 1));
  if (!p) caml_failwith("mmo_gpu: out of memory");
  for (i = 0; i < n; ++i) p[i] = Int_val(Field(a, i));
  return p;
}

/* Wosize of a flat float array is its length in doubles on 64-bit hosts */
static int n_floats(value a) { return (int)(Wosize_val(a) * sizeof(value) / sizeof(double)); }

CAMLprim value mmo_ocaml_create(value device) {
  CAMLparam1(device);
  CAMLlocal1(v);
  mmo_ctx *c = NULL;
  if (mmo_ctx_create(Int_val(device), &c) != MMO_OK) caml_failwith(mmo_last_error(NULL));
  v = caml_alloc_custom(&ctx_ops, sizeof(mmo_ctx *), 0, 1);
  Ctx_val(v) = c;
  CAMLreturn(v);
}

CAMLprim value mmo_ocaml_set_physics(value ctx, value diel, value mix, value inter, value intra) {
  CAMLparam5(ctx, diel, mix, inter, intra);
  mmo_ctx *c = Ctx_val(ctx);
  check(c, mmo_set_physics(c, Int_val(diel), Int_val(mix), Int_val(inter), Int_val(intra)));
  CAMLreturn(Val_unit);
}

CAMLprim value mmo_ocaml_set_protein(value ctx, value xs, value ys, value zs, value q,
                                     value anum) {
  CAMLparam5(ctx, xs, ys, zs, q);
  CAMLxparam1(anum);
  mmo_ctx *c = Ctx_val(ctx);
  int *an = c_ints(anum);
  int rc = mmo_set_protein(c, n_floats(xs), Doubles(xs), Doubles(ys), Doubles(zs), Doubles(q), an);
  free(an);
  check(c, rc);
  CAMLreturn(Val_unit);
}

CAMLprim value mmo_ocaml_set_protein_byte(value *argv, int argn) {
  (void)argn;
  return mmo_ocaml_set_protein(argv[0], argv[1], argv[2], argv[3], argv[4], argv[5]);
}

/* interacting: n*n bytes; bond_lr: 2*nrb; goff: nrb+1; gatoms: flat groups */
CAMLprim value mmo_ocaml_set_ligand(value ctx, value xs, value ys, value zs, value q,
                                    value anum, value interacting, value bond_lr, value goff,
                                    value gatoms) {
  CAMLparam5(ctx, xs, ys, zs, q);
  CAMLxparam5(anum, interacting, bond_lr, goff, gatoms);
  mmo_ctx *c = Ctx_val(ctx);
  int *an = c_ints(anum), *bl = c_ints(bond_lr), *go = c_ints(goff), *ga = c_ints(gatoms);
  int nrb = (int)(Wosize_val(bond_lr) / 2);
  int rc = mmo_set_ligand(c, n_floats(xs), Doubles(xs), Doubles(ys), Doubles(zs), Doubles(q),
                          an, (const uint8_t *)Bytes_val(interacting), nrb, bl, go, ga);
  free(an);
  free(bl);
  free(go);
  free(ga);
  check(c, rc);
  CAMLreturn(Val_unit);
}

CAMLprim value mmo_ocaml_set_ligand_byte(value *argv, int argn) {
  (void)argn;
  return mmo_ocaml_set_ligand(argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6],
                              argv[7], argv[8], argv[9]);
}

CAMLprim value mmo_ocaml_ene_inter(value ctx, value xs, value ys, value zs, value q,
                                   value anum) {
  CAMLparam5(ctx, xs, ys, zs, q);
  CAMLxparam1(anum);
  mmo_ctx *c = Ctx_val(ctx);
  double e = 0.0;
  int *an = c_ints(anum);
  int rc = mmo_ene_inter(c, n_floats(xs), Doubles(xs), Doubles(ys), Doubles(zs), Doubles(q), an,
                         &e);
  free(an);
  check(c, rc);
  CAMLreturn(caml_copy_double(e));
}

CAMLprim value mmo_ocaml_ene_inter_byte(value *argv, int argn) {
  (void)argn;
  return mmo_ocaml_ene_inter(argv[0], argv[1], argv[2], argv[3], argv[4], argv[5]);
}

/* Mol.ene_inter_UFF_shifted_bst_components (mol.ml:920-957): (elec, vdW) */
CAMLprim value mmo_ocaml_ene_inter_parts(value ctx, value xs, value ys, value zs, value q,
                                         value anum) {
  CAMLparam5(ctx, xs, ys, zs, q);
  CAMLxparam1(anum);
  CAMLlocal1(res);
  mmo_ctx *c = Ctx_val(ctx);
  double el = 0.0, vdw = 0.0;
  int *an = c_ints(anum);
  int rc = mmo_ene_inter_parts(c, n_floats(xs), Doubles(xs), Doubles(ys), Doubles(zs), Doubles(q),
                               an, &el, &vdw);
  free(an);
  check(c, rc);
  res = caml_alloc_tuple(2);
  Store_field(res, 0, caml_copy_double(el));
  Store_field(res, 1, caml_copy_double(vdw));
  CAMLreturn(res);
}

CAMLprim value mmo_ocaml_ene_inter_parts_byte(value *argv, int argn) {
  (void)argn;
  return mmo_ocaml_ene_inter_parts(argv[0], argv[1], argv[2], argv[3], argv[4], argv[5]);
}

CAMLprim value mmo_ocaml_ene_intra(value ctx, value xs, value ys, value zs) {
  CAMLparam4(ctx, xs, ys, zs);
  mmo_ctx *c = Ctx_val(ctx);
  double e = 0.0;
  check(c, mmo_ene_intra(c, Doubles(xs), Doubles(ys), Doubles(zs), &e));
  CAMLreturn(caml_copy_double(e));
}

/* dofs: B*(6+nrb) floats (Optim.config rows, src/optim.ml:19-22); returns
 * (energies, gradients or [||], statuses) */
CAMLprim value mmo_ocaml_score_poses(value ctx, value dofs, value nd, value flags) {
  CAMLparam4(ctx, dofs, nd, flags);
  CAMLlocal4(res, e_arr, g_arr, s_arr);
  mmo_ctx *c = Ctx_val(ctx);
  const int ndof = Int_val(nd), fl = Int_val(flags);
  const int total = n_floats(dofs), B = ndof > 0 ? total / ndof : 0;
  float *d = (float *)malloc(sizeof(float) * (total ? total : 1));
  double *E = (double *)malloc(sizeof(double) * (B ? B : 1));
  float *G = (fl & MMO_F_GRAD) ? (float *)malloc(sizeof(float) * (total ? total : 1)) : NULL;
  int *st = (int *)malloc(sizeof(int) * (B ? B : 1)), i, rc;
  for (i = 0; i < total; ++i) d[i] = (float)Double_flat_field(dofs, i);
  rc = mmo_score_poses(c, B, d, fl, E, G, st);
  if (rc != MMO_OK) {
    free(d);
    free(E);
    free(G);
    free(st);
    check(c, rc);
  }
  e_arr = caml_alloc_float_array(B);
  for (i = 0; i < B; ++i) Store_double_flat_field(e_arr, i, E[i]);
  g_arr = caml_alloc_float_array(G ? total : 0);
  if (G)
    for (i = 0; i < total; ++i) Store_double_flat_field(g_arr, i, (double)G[i]);
  s_arr = caml_alloc(B, 0);
  for (i = 0; i < B; ++i) Store_field(s_arr, i, Val_int(st[i]));
  res = caml_alloc_tuple(3);
  Store_field(res, 0, e_arr);
  Store_field(res, 1, g_arr);
  Store_field(res, 2, s_arr);
  free(d);
  free(E);
  free(G);
  free(st);
  CAMLreturn(res);
}

/* one Optim.config: E_inter + E_intra, raising Mol.Too_long as
 * Optim.apply_config does */
CAMLprim value mmo_ocaml_score_config(value ctx, value conf) {
  CAMLparam2(ctx, conf);
  mmo_ctx *c = Ctx_val(ctx);
  const int n = n_floats(conf);
  float d[6 + 32];
  double E = 0.0;
  int st = 0, i;
  if (n > 6 + 32) caml_failwith("mmo_gpu: more than 32 rotatable bonds");
  for (i = 0; i < n; ++i) d[i] = (float)Double_flat_field(conf, i);
  check(c, mmo_score_poses(c, 1, d, MMO_F_INTER | MMO_F_INTRA, &E, NULL, &st));
  if (st & MMO_S_TOO_LONG) {
    const value *exn = caml_named_value("Mol.Too_long");
    if (exn) caml_raise_constant(*exn);
    caml_failwith("Mol.Too_long");
  }
  CAMLreturn(caml_copy_double(E));
}

/* Lds.pre_calculate_FF_components_grid on the GPU (mmo_build_grids):
 * lattice = [| step; origin x; y; z |], dims = [| nx; ny; nz |], the types'
 * atomic numbers and charges (Mol.get_all_vdW_elec_types), mask =
 * [| cx; cy; cz; radius |] (radius <= 0: no mask), max_E. */
CAMLprim value mmo_ocaml_build_grids(value ctx, value lattice, value dims, value type_anum,
                                     value type_q, value mask, value max_e) {
  CAMLparam5(ctx, lattice, dims, type_anum, type_q);
  CAMLxparam2(mask, max_e);
  mmo_ctx *c = Ctx_val(ctx);
  mmo_grid_spec sp;
  int *ta = c_ints(type_anum), i, rc;
  sp.step = Double_flat_field(lattice, 0);
  for (i = 0; i < 3; ++i) {
    sp.origin[i] = Double_flat_field(lattice, 1 + i);
    sp.mask_center[i] = Double_flat_field(mask, i);
  }
  sp.nx = Int_val(Field(dims, 0));
  sp.ny = Int_val(Field(dims, 1));
  sp.nz = Int_val(Field(dims, 2));
  sp.mask_radius = Double_flat_field(mask, 3);
  sp.max_E = Double_val(max_e);
  sp.ntypes = (int)Wosize_val(type_anum);
  sp.type_anum = ta;
  sp.type_q = Doubles(type_q);
  rc = mmo_build_grids(c, &sp, NULL);
  free(ta);
  check(c, rc);
  CAMLreturn(Val_unit);
}

CAMLprim value mmo_ocaml_build_grids_byte(value *argv, int argn) {
  (void)argn;
  return mmo_ocaml_build_grids(argv[0], argv[1], argv[2], argv[3], argv[4], argv[5], argv[6]);
}

/* Mol.ene_inter_UFF_interp grid ff_comps on the context's grids */
CAMLprim value mmo_ocaml_ene_inter_grid(value ctx, value xs, value ys, value zs, value q,
                                        value anum) {
  CAMLparam5(ctx, xs, ys, zs, q);
  CAMLxparam1(anum);
  mmo_ctx *c = Ctx_val(ctx);
  double e = 0.0;
  int st = 0;
  int *an = c_ints(anum);
  int rc = mmo_ene_inter_grid(c, n_floats(xs), Doubles(xs), Doubles(ys), Doubles(zs), Doubles(q),
                              an, &e, &st);
  free(an);
  check(c, rc);
  CAMLreturn(caml_copy_double(e));
}

CAMLprim value mmo_ocaml_ene_inter_grid_byte(value *argv, int argn) {
  (void)argn;
  return mmo_ocaml_ene_inter_grid(argv[0], argv[1], argv[2], argv[3], argv[4], argv[5]);
}
