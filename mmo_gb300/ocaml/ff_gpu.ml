(* ff_gpu.ml -- GPU drop-ins for MMO's force-field scoring closures.
 *
 * Replaces, in src/lds.ml, [ff0 prot] (Mol.ene_inter_UFF_shifted_bst prot_bst
 * prot, lines 1952-1967) and [ene_intra_builder UFF_NB] (lines 702-712), and
 * gives a batched scorer with the analytic gradient for the NLopt objective
 * (lines 1246-1274) in place of approx_local_gradient (lines 1118-1136).
 * Contexts are created on first use, so after parany's fork. *)

type ctx

external create : int -> ctx = "mmo_ocaml_create"
external set_physics : ctx -> int -> int -> int -> int -> unit = "mmo_ocaml_set_physics"
external set_protein_raw :
  ctx -> float array -> float array -> float array -> float array -> int array -> unit
  = "mmo_ocaml_set_protein_byte" "mmo_ocaml_set_protein"
external set_ligand_raw :
  ctx -> float array -> float array -> float array -> float array -> int array -> Bytes.t ->
  int array -> int array -> int array -> unit
  = "mmo_ocaml_set_ligand_byte" "mmo_ocaml_set_ligand"
external ene_inter_raw :
  ctx -> float array -> float array -> float array -> float array -> int array -> float
  = "mmo_ocaml_ene_inter_byte" "mmo_ocaml_ene_inter"
external ene_inter_parts_raw :
  ctx -> float array -> float array -> float array -> float array -> int array -> float * float
  = "mmo_ocaml_ene_inter_parts_byte" "mmo_ocaml_ene_inter_parts"
external ene_intra_raw : ctx -> float array -> float array -> float array -> float
  = "mmo_ocaml_ene_intra"
external score_poses_raw :
  ctx -> float array -> int -> int -> float array * float array * int array
  = "mmo_ocaml_score_poses"
external score_config : ctx -> float array -> float = "mmo_ocaml_score_config"
external build_grids_raw :
  ctx -> float array -> int array -> int array -> float array -> float array -> float -> unit
  = "mmo_ocaml_build_grids_byte" "mmo_ocaml_build_grids"
external ene_inter_grid_raw :
  ctx -> float array -> float array -> float array -> float array -> int array -> float
  = "mmo_ocaml_ene_inter_grid_byte" "mmo_ocaml_ene_inter_grid"

let () = Callback.register_exception "Mol.Too_long" Mol.Too_long

let f_inter = 1
let f_intra = 2
let f_grad = 4
let f_recenter = 8

let device () =
  match Sys.getenv_opt "MMO_GPU_DEVICE" with
  | Some d -> int_of_string d
  | None -> 0

(* one context per process, created lazily (after the fork) *)
let the_ctx = ref None
let get_ctx () =
  match !the_ctx with
  | Some c -> c
  | None -> let c = create (device ()) in the_ctx := Some c; c

let set_protein ctx (p: Mol.t) =
  set_protein_raw ctx p.Mol.xs p.Mol.ys p.Mol.zs p.Mol.q_a p.Mol.elt_a

let set_ligand ctx (l: Mol.t) =
  let n = Array.length l.Mol.xs in
  let inter = Bytes.make (n * n) '\000' in
  Array.iteri (fun i row ->
      Array.iteri (fun j b -> if b then Bytes.set inter (i * n + j) '\001') row
    ) l.Mol.interacting_a;
  let nrb = Array.length l.Mol.rbonds_a in
  let bond_lr = Array.make (2 * nrb) 0 in
  Array.iteri (fun t b ->
      bond_lr.(2 * t) <- b.Bond.left;
      bond_lr.(2 * t + 1) <- b.Bond.right
    ) l.Mol.rbonds_a;
  let goff = Array.make (nrb + 1) 0 in
  Array.iteri (fun t g -> goff.(t + 1) <- goff.(t) + Array.length g) l.Mol.rgroups_a;
  let gatoms = Array.concat (Array.to_list l.Mol.rgroups_a) in
  set_ligand_raw ctx l.Mol.xs l.Mol.ys l.Mol.zs l.Mol.q_a l.Mol.elt_a inter bond_lr goff gatoms

(* drop-in for [ff0 prot]: Mol.t -> float *)
let ene_inter_builder (prot: Mol.t) =
  let ready = ref false in
  fun (lig: Mol.t) ->
    let c = get_ctx () in
    if not !ready then (set_protein c prot; ready := true);
    ene_inter_raw c lig.Mol.xs lig.Mol.ys lig.Mol.zs lig.Mol.q_a lig.Mol.elt_a

(* drop-in for [Mol.ene_inter_UFF_shifted_bst_components prot_bst prot]:
   Mol.t -> Mol.ele_vdW (mol.ml:920-957) *)
let ene_inter_components_builder (prot: Mol.t) =
  let ready = ref false in
  fun (lig: Mol.t) ->
    let c = get_ctx () in
    if not !ready then (set_protein c prot; ready := true);
    let el, vdw =
      ene_inter_parts_raw c lig.Mol.xs lig.Mol.ys lig.Mol.zs lig.Mol.q_a lig.Mol.elt_a in
    { Mol.sum_elec = el; sum_vdW = vdw }

(* drop-in for [ene_intra_builder UFF_NB] *)
let ene_intra_builder tweak_rbonds (centered_lig: Mol.t) =
  let ready = ref false in
  let setup () =
    let c = get_ctx () in
    if not !ready then (set_ligand c centered_lig; ready := true);
    c in
  if tweak_rbonds && Array.length centered_lig.Mol.rbonds_a > 0 then
    (fun (lig: Mol.t) -> ene_intra_raw (setup ()) lig.Mol.xs lig.Mol.ys lig.Mol.zs)
  else
    let e = lazy (let c = setup () in
                  ene_intra_raw c centered_lig.Mol.xs centered_lig.Mol.ys centered_lig.Mol.zs) in
    (fun _lig -> Lazy.force e)

(* energies and analytic gradients of many Optim.config rows at once *)
let score_configs ?(recenter = false) (confs: float array array) =
  let c = get_ctx () in
  let nd = if Array.length confs = 0 then 0 else Array.length confs.(0) in
  let flat = Array.concat (Array.to_list confs) in
  let flags = f_inter lor f_intra lor f_grad lor (if recenter then f_recenter else 0) in
  let e, g, st = score_poses_raw c flat nd flags in
  (e, Array.init (Array.length e) (fun b -> Array.sub g (b * nd) nd), st)

(* drop-in for [ff1] of lds.ml:1963-1975: the per-type grids of [types]
 * (Mol.get_all_vdW_elec_types's (anum, charge) pairs, in type order) built on
 * the GPU over [grid] (Grid.from_box; lowest point at the origin of the
 * simulation box) with the ROI mask of Lds.bitmask_ROI_only, then
 * Mol.ene_inter_UFF_interp grid ff_comps : Mol.t -> float *)
let ene_inter_interp_builder (prot: Mol.t) (grid: Grid.t) (types: (int * float) array)
    (roi_center: float * float * float) (roi_out_radius: float) =
  let ready = ref false in
  fun (lig: Mol.t) ->
    let c = get_ctx () in
    if not !ready then begin
      set_protein c prot;
      let cx, cy, cz = roi_center in
      build_grids_raw c [| grid.Grid.step; 0.0; 0.0; 0.0 |]
        [| grid.Grid.x_dim; grid.Grid.y_dim; grid.Grid.z_dim |]
        (Array.map fst types) (Array.map snd types)
        [| cx; cy; cz; roi_out_radius +. 2.0 *. 12.0 |] 100_000.0;
      ready := true
    end;
    ene_inter_grid_raw c lig.Mol.xs lig.Mol.ys lig.Mol.zs lig.Mol.q_a lig.Mol.elt_a
