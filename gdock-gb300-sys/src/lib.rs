//! FFI bindings to `libgdock_gb300`, the GB300 engine that replaces gdock's
//! population fitness evaluation and FCC clustering.
//!
//! The declarations mirror `include/gdock_gb300.h` one for one: every
//! `extern "C"` entry point with its arguments in order, every `#[repr(C)]`
//! struct with its fields in order.  A CPU test of the library's repository
//! (`tests/test_ffi_crate.py`) parses both files and checks that they agree.
//!
//! On top of the raw calls sit the small pieces every call site needs:
//! [`PackedAtoms`] (a molecule as the structure-of-arrays `gd_atoms` reads),
//! [`element_class`], [`pack_name`], [`last_error`], and owning handles
//! ([`Context`], [`Complex`]) that release their objects on drop.
#![allow(non_camel_case_types)]

use std::ffi::CStr;
use std::marker::{PhantomData, PhantomPinned};
use std::os::raw::{c_char, c_int, c_void};

// ---------------------------------------------------------------- constants

pub const GD_ABI_VERSION: i32 = 1;

/// `gd_status`: every call returns one (a C enum, passed as an int).
pub type gd_status = c_int;
pub const GD_OK: gd_status = 0;
pub const GD_ERR_INVALID_ARG: gd_status = 1;
pub const GD_ERR_OOM: gd_status = 2;
pub const GD_ERR_CUDA: gd_status = 3;
pub const GD_ERR_TIMEOUT: gd_status = 4;
pub const GD_ERR_CAPACITY: gd_status = 5;
pub const GD_ERR_STATE: gd_status = 6;

/// `gd_precision`: the plain FP64 form or the FP32 form.
pub type gd_precision = c_int;
pub const GD_PREC_F64: gd_precision = 0;
pub const GD_PREC_F32: gd_precision = 1;

/// Element classes of `gd_atoms.element` (src/structure.rs:241-256).
pub const GD_ELEM_OTHER: u8 = 0;
pub const GD_ELEM_H: u8 = 1;
pub const GD_ELEM_C: u8 = 2;
pub const GD_ELEM_N: u8 = 3;
pub const GD_ELEM_O: u8 = 4;
pub const GD_ELEM_S: u8 = 5;

/// Knobs of `gd_context_set_tuning` / `gd_context_get_tuning`.
pub const GD_TUNE_F32_SLOTS: i32 = 0;
pub const GD_TUNE_SPLIT: i32 = 1;
pub const GD_TUNE_FAULT: i32 = 2;
pub const GD_TUNE_FCC: i32 = 3;
pub const GD_TUNE_CONTACTS: i32 = 4;
pub const GD_TUNE_RPARTS: i32 = 5;
/// Read-only values of `gd_context_get_tuning`.
pub const GD_INFO_LAST_FCC: i32 = 16;
pub const GD_INFO_LAST_CONTACTS: i32 = 17;

pub const GD_AUTOTUNE_CANDIDATES: usize = 6;
pub const GD_EVAL_COUNTS: usize = 7;

/// Job states of the server.
pub const GD_JOB_QUEUED: i32 = 0;
pub const GD_JOB_RUNNING: i32 = 1;
pub const GD_JOB_DONE: i32 = 2;
pub const GD_JOB_FAILED: i32 = 3;

// ------------------------------------------------------------ opaque types

macro_rules! opaque {
    ($name:ident) => {
        #[repr(C)]
        pub struct $name {
            _p: [u8; 0],
            _m: PhantomData<(*mut u8, PhantomPinned)>,
        }
    };
}
opaque!(gd_context);
opaque!(gd_complex);
opaque!(gd_evaluator);
opaque!(gd_server);

// ----------------------------------------------------------------- structs

/// One molecule as structure-of-arrays (gdock's `Atom` fields the GPU reads,
/// src/structure.rs:27-49).  Pointers must stay valid for the call.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct gd_atoms {
    pub n: i32,
    pub x: *const f64,
    pub y: *const f64,
    pub z: *const f64,
    pub epsilon: *const f64,
    pub rmin2: *const f64,
    pub charge: *const f64,
    pub vdw_radius: *const f64,
    pub serial: *const i32,
    pub resseq: *const i16,
    pub chain: *const u8,
    pub element: *const u8,
    pub is_ca: *const u8,
}

/// `EnergyWeights` (src/constants.rs:28-56).
#[repr(C)]
#[derive(Clone, Copy, Debug, PartialEq)]
pub struct gd_weights {
    pub vdw: f64,
    pub elec: f64,
    pub desolv: f64,
    pub air: f64,
}

/// The six fields `Chromosome::fitness` writes (src/chromosome.rs:111-127).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct gd_pose_energy {
    pub fitness: f64,
    pub vdw: f64,
    pub elec: f64,
    pub desolv: f64,
    pub air: f64,
    pub restraint_penalty: f64,
}

/// `ClusteringConfig` (src/clustering.rs:14-35).
#[repr(C)]
#[derive(Clone, Copy, Debug, PartialEq)]
pub struct gd_cluster_cfg {
    pub contact_distance: f64,
    pub fcc_cutoff: f64,
    pub strictness: f64,
    pub min_cluster_size: i32,
}

impl Default for gd_cluster_cfg {
    fn default() -> Self {
        gd_cluster_cfg { contact_distance: 5.0, fcc_cutoff: 0.60, strictness: 0.75, min_cluster_size: 4 }
    }
}

/// A pose's rotation and translation as the host precomputes them
/// (`gd_make_frames`).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct gd_pose_frame {
    pub ca: f64,
    pub sa: f64,
    pub cb: f64,
    pub sb: f64,
    pub cg: f64,
    pub sg: f64,
    pub m01: f64,
    pub m02: f64,
    pub m11: f64,
    pub m12: f64,
    pub dx: f64,
    pub dy: f64,
    pub dz: f64,
    pub pad: [f64; 3],
}

/// `evaluator::Metrics` (src/evaluator.rs:29-35).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct gd_dock_metrics {
    pub rmsd: f64,
    pub irmsd: f64,
    pub fnat: f64,
    pub dockq: f64,
}

/// GA settings (src/constants.rs:2-16, src/chromosome.rs:64-71).
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct gd_ga_cfg {
    pub pop_size: i32,
    pub elitism: i32,
    pub tournament_size: i32,
    pub crossover_rate: f64,
    pub mutation_rate: f64,
    pub max_displacement: f64,
    pub rot_sigma: f64,
    pub trans_sigma: f64,
    pub max_generations: i32,
    pub early_stopping: i32,
    pub convergence_threshold: f64,
    pub convergence_window: i32,
    pub seed: u64,
    pub hof_max_size: i32,
    pub hof_top_k: i32,
}

/// One Hall of Fame entry (src/commands/run.rs:64-73).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct gd_hof_entry {
    pub genes: [f64; 6],
    pub fitness: f64,
    pub generation: i32,
    pub pad: i32,
}

/// Per-generation DockQ outputs of `gd_ga_run`.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct gd_ga_metrics {
    pub evaluators: *const *mut gd_evaluator,
    pub best: *mut gd_dock_metrics,
    pub mean_dockq: *mut f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct gd_server_cfg {
    pub max_slots: i32,
    pub hbm_budget: u64,
    pub ga: gd_ga_cfg,
    pub precision: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct gd_job_result {
    pub status: i32,
    pub error: i32,
    pub generations: i32,
    pub latency_s: f64,
    pub queue_s: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct gd_server_stats {
    pub completed: i64,
    pub queued: i64,
    pub resident: i64,
    pub generations_run: i64,
    pub poses_scored: i64,
    pub device_bytes: u64,
    pub latency_p50_s: f64,
    pub latency_p99_s: f64,
    pub latency_max_s: f64,
    pub gpu_busy_s: f64,
    pub elapsed_s: f64,
}

// ------------------------------------------------------------- entry points

extern "C" {
    pub fn gd_abi_version() -> i32;
    pub fn gd_status_string(s: gd_status) -> *const c_char;

    pub fn gd_context_create(device: i32, hbm_budget_bytes: u64, out: *mut *mut gd_context) -> gd_status;
    pub fn gd_context_destroy(ctx: *mut gd_context) -> gd_status;
    pub fn gd_context_set_tuning(ctx: *mut gd_context, knob: i32, value: i32) -> gd_status;
    pub fn gd_autotune_f32(cx: *mut gd_complex, d_frames: *const gd_pose_frame, n: i32, max_displacement: f64,
                           d_out: *mut gd_pose_energy, stream: *mut c_void, rates: *mut f64,
                           best: *mut i32) -> gd_status;
    pub fn gd_context_get_tuning(ctx: *const gd_context, knob: i32) -> i32;
    pub fn gd_last_error(ctx: *const gd_context) -> *const c_char;
    pub fn gd_context_bytes_in_use(ctx: *const gd_context) -> u64;

    pub fn gd_complex_create(ctx: *mut gd_context, receptor: *const gd_atoms, ligand: *const gd_atoms,
                             restraint_pairs: *const i32, n_pairs: i32, w: *const gd_weights,
                             out: *mut *mut gd_complex) -> gd_status;
    pub fn gd_complex_destroy(cx: *mut gd_complex) -> gd_status;
    pub fn gd_complex_num_restraints(cx: *const gd_complex) -> i32;
    pub fn gd_complex_set_weights(cx: *mut gd_complex, w: *const gd_weights) -> gd_status;

    pub fn gd_make_frames(genes: *const f64, n: i32, frames: *mut gd_pose_frame) -> gd_status;
    pub fn gd_score_poses(cx: *mut gd_complex, genes: *const f64, n: i32, prec: gd_precision,
                          out: *mut gd_pose_energy) -> gd_status;
    pub fn gd_score_frames_device(cx: *mut gd_complex, d_frames: *const gd_pose_frame, n: i32, prec: gd_precision,
                                  max_displacement: f64, d_out: *mut gd_pose_energy,
                                  stream: *mut c_void) -> gd_status;
    pub fn gd_score_frames_device_noalloc(cx: *mut gd_complex, d_frames: *const gd_pose_frame, n: i32,
                                          max_displacement: f64, d_out: *mut gd_pose_energy,
                                          stream: *mut c_void) -> gd_status;
    pub fn gd_sync(ctx: *mut gd_context) -> gd_status;
    pub fn gd_score_models(cx: *mut gd_complex, lig_xyz: *const f64, n_models: i32, prec: gd_precision,
                           out: *mut gd_pose_energy) -> gd_status;

    pub fn gd_pose_contacts(cx: *mut gd_complex, genes: *const f64, n: i32, keys: *mut i64, cap: i64,
                            offsets: *mut i64) -> gd_status;
    pub fn gd_cluster(cx: *mut gd_complex, genes: *const f64, n: i32, cfg: *const gd_cluster_cfg,
                      n_clusters: *mut i32, centers: *mut i32, sizes: *mut i32, members: *mut i32) -> gd_status;
    pub fn gd_cluster_sets(ctx: *mut gd_context, keys: *const i64, offsets: *const i64, n: i32,
                           cfg: *const gd_cluster_cfg, n_clusters: *mut i32, centers: *mut i32, sizes: *mut i32,
                           members: *mut i32) -> gd_status;

    pub fn gd_evaluator_create(cx: *mut gd_complex, reference: *const gd_atoms, rec_names: *const u32,
                               lig_names: *const u32, ref_names: *const u32,
                               out: *mut *mut gd_evaluator) -> gd_status;
    pub fn gd_evaluator_destroy(ev: *mut gd_evaluator) -> gd_status;
    pub fn gd_evaluator_counts(ev: *const gd_evaluator, counts: *mut i64) -> gd_status;
    pub fn gd_evaluate_poses(ev: *mut gd_evaluator, genes: *const f64, n: i32, out: *mut gd_dock_metrics)
                             -> gd_status;
    pub fn gd_evaluate_frames_device(ev: *mut gd_evaluator, d_frames: *const gd_pose_frame, n: i32,
                                     d_out: *mut gd_dock_metrics, stream: *mut c_void) -> gd_status;

    pub fn gd_ga_default_cfg(cfg: *mut gd_ga_cfg) -> gd_status;
    pub fn gd_ga_draw(cfg: *const gd_ga_cfg, seed: u64, generations: i32, init_genes: *mut f64, tour: *mut i32,
                      perm: *mut i32, cross_u: *mut f64, mut_u: *mut f64, mut_z: *mut f64) -> gd_status;
    pub fn gd_ga_run(ctx: *mut gd_context, complexes: *const *mut gd_complex, jobs: i32, cfg: *const gd_ga_cfg,
                     prec: gd_precision, use_graph: i32, out_genes: *mut f64, out_energies: *mut gd_pose_energy,
                     out_generations: *mut i32, out_history: *mut f64, out_hof: *mut gd_hof_entry,
                     out_hof_count: *mut i32, metrics: *const gd_ga_metrics) -> gd_status;

    pub fn gd_server_default_cfg(cfg: *mut gd_server_cfg) -> gd_status;
    pub fn gd_server_create(ctx: *mut gd_context, cfg: *const gd_server_cfg, out: *mut *mut gd_server) -> gd_status;
    pub fn gd_server_destroy(s: *mut gd_server) -> gd_status;
    pub fn gd_server_submit(s: *mut gd_server, receptor: *const gd_atoms, ligand: *const gd_atoms,
                            restraint_pairs: *const i32, n_pairs: i32, w: *const gd_weights, seed: u64,
                            job_id: *mut i64) -> gd_status;
    pub fn gd_server_step(s: *mut gd_server, resident_jobs: *mut i32) -> gd_status;
    pub fn gd_server_start(s: *mut gd_server) -> gd_status;
    pub fn gd_server_stop(s: *mut gd_server) -> gd_status;
    pub fn gd_server_wait(s: *mut gd_server, job_id: i64, timeout_s: f64, status: *mut i32) -> gd_status;
    pub fn gd_server_result(s: *mut gd_server, job_id: i64, res: *mut gd_job_result, genes: *mut f64,
                            energies: *mut gd_pose_energy, history: *mut f64) -> gd_status;
    pub fn gd_server_hall_of_fame(s: *mut gd_server, job_id: i64, entries: *mut gd_hof_entry, cap: i32,
                                  count: *mut i32) -> gd_status;
    pub fn gd_server_release(s: *mut gd_server, job_id: i64) -> gd_status;
    pub fn gd_server_get_stats(s: *mut gd_server, out: *mut gd_server_stats) -> gd_status;
}

// ------------------------------------------------------------------ helpers

/// The fields of gdock's `structure::Atom` that [`PackedAtoms`] reads.  The
/// integration implements it for `Atom` (a one-line accessor per field).
pub trait AtomFields {
    fn x(&self) -> f64;
    fn y(&self) -> f64;
    fn z(&self) -> f64;
    fn epsilon(&self) -> f64;
    fn rmin2(&self) -> f64;
    fn charge(&self) -> f64;
    fn vdw_radius(&self) -> f64;
    fn serial(&self) -> i32;
    fn resseq(&self) -> i16;
    fn chainid(&self) -> char;
    fn element(&self) -> &str;
    fn name(&self) -> &str;
}

/// Element column -> `GD_ELEM_*`, on the trimmed text as gdock matches it
/// (src/fitness.rs:129-138, src/clustering.rs:67-70).
pub fn element_class(element: &str) -> u8 {
    match element.trim() {
        "H" => GD_ELEM_H,
        "C" => GD_ELEM_C,
        "N" => GD_ELEM_N,
        "O" => GD_ELEM_O,
        "S" => GD_ELEM_S,
        _ => GD_ELEM_OTHER,
    }
}

/// A trimmed atom name (at most 4 characters) packed little-endian into a
/// `u32`, byte k = character k, as `gd_evaluator_create` reads names.
pub fn pack_name(name: &str) -> u32 {
    name.trim().bytes().take(4).enumerate().fold(0u32, |v, (k, b)| v | (b as u32) << (8 * k))
}

/// One molecule packed as the structure-of-arrays the ABI reads.  The
/// vectors own the data; [`PackedAtoms::view`] points into them.
#[derive(Clone, Debug, Default)]
pub struct PackedAtoms {
    pub x: Vec<f64>,
    pub y: Vec<f64>,
    pub z: Vec<f64>,
    pub epsilon: Vec<f64>,
    pub rmin2: Vec<f64>,
    pub charge: Vec<f64>,
    pub vdw_radius: Vec<f64>,
    pub serial: Vec<i32>,
    pub resseq: Vec<i16>,
    pub chain: Vec<u8>,
    pub element: Vec<u8>,
    pub is_ca: Vec<u8>,
    pub names: Vec<u32>,
}

impl PackedAtoms {
    pub fn new<'a, A: AtomFields + 'a, I: IntoIterator<Item = &'a A>>(atoms: I) -> Self {
        let mut p = PackedAtoms::default();
        for a in atoms {
            p.x.push(a.x());
            p.y.push(a.y());
            p.z.push(a.z());
            p.epsilon.push(a.epsilon());
            p.rmin2.push(a.rmin2());
            p.charge.push(a.charge());
            p.vdw_radius.push(a.vdw_radius());
            p.serial.push(a.serial());
            p.resseq.push(a.resseq());
            p.chain.push(a.chainid() as u8);
            p.element.push(element_class(a.element()));
            p.is_ca.push((a.name().trim() == "CA") as u8);
            p.names.push(pack_name(a.name()));
        }
        p
    }

    pub fn len(&self) -> usize {
        self.x.len()
    }

    pub fn is_empty(&self) -> bool {
        self.x.is_empty()
    }

    /// The `gd_atoms` view of the vectors (valid while `self` is neither
    /// moved nor changed).
    pub fn view(&self) -> gd_atoms {
        gd_atoms {
            n: self.x.len() as i32,
            x: self.x.as_ptr(),
            y: self.y.as_ptr(),
            z: self.z.as_ptr(),
            epsilon: self.epsilon.as_ptr(),
            rmin2: self.rmin2.as_ptr(),
            charge: self.charge.as_ptr(),
            vdw_radius: self.vdw_radius.as_ptr(),
            serial: self.serial.as_ptr(),
            resseq: self.resseq.as_ptr(),
            chain: self.chain.as_ptr(),
            element: self.element.as_ptr(),
            is_ca: self.is_ca.as_ptr(),
        }
    }
}

/// The message of the context's last failing call.
pub fn last_error(ctx: *const gd_context) -> String {
    unsafe {
        let p = gd_last_error(ctx);
        if p.is_null() {
            return String::new();
        }
        CStr::from_ptr(p).to_string_lossy().into_owned()
    }
}

/// A failed call: its status and the context's message.
#[derive(Clone, Debug)]
pub struct Error {
    pub status: gd_status,
    pub message: String,
}

impl std::fmt::Display for Error {
    fn fmt(&self, f: &mut std::fmt::Formatter<'_>) -> std::fmt::Result {
        let s = unsafe { CStr::from_ptr(gd_status_string(self.status)) }.to_string_lossy();
        write!(f, "gdock_gb300: {} ({})", s, self.message)
    }
}

impl std::error::Error for Error {}

pub fn check(ctx: *const gd_context, status: gd_status) -> Result<(), Error> {
    if status == GD_OK {
        Ok(())
    } else {
        Err(Error { status, message: last_error(ctx) })
    }
}

/// An owned context on one CUDA device.  A context belongs to one host
/// thread at a time: it may move between threads but is not shared.
pub struct Context {
    pub raw: *mut gd_context,
}

unsafe impl Send for Context {}

impl Context {
    pub fn new(device: i32, hbm_budget_bytes: u64) -> Result<Context, Error> {
        let mut raw = std::ptr::null_mut();
        let st = unsafe { gd_context_create(device, hbm_budget_bytes, &mut raw) };
        if st != GD_OK {
            return Err(Error { status: st, message: String::from("gd_context_create") });
        }
        Ok(Context { raw })
    }
}

impl Drop for Context {
    fn drop(&mut self) {
        unsafe {
            gd_context_destroy(self.raw);
        }
    }
}

/// An owned complex (receptor, positioned ligand, restraints, weights)
/// uploaded to its context's device.  It must be dropped before its context.
pub struct Complex {
    pub raw: *mut gd_complex,
    ctx: *mut gd_context,
}

unsafe impl Send for Complex {}

impl Complex {
    /// `restraint_pairs` are (receptor resseq, ligand resseq) pairs, as
    /// `create_restraints_from_pairs` takes them.
    pub fn new(ctx: &Context, receptor: &PackedAtoms, ligand: &PackedAtoms, restraint_pairs: &[(i32, i32)],
               weights: &gd_weights) -> Result<Complex, Error> {
        let flat: Vec<i32> = restraint_pairs.iter().flat_map(|&(r, l)| [r, l]).collect();
        let (rv, lv) = (receptor.view(), ligand.view());
        let mut raw = std::ptr::null_mut();
        let st = unsafe {
            gd_complex_create(ctx.raw, &rv, &lv, if flat.is_empty() { std::ptr::null() } else { flat.as_ptr() },
                              restraint_pairs.len() as i32, weights, &mut raw)
        };
        check(ctx.raw, st)?;
        Ok(Complex { raw, ctx: ctx.raw })
    }

    /// `Population::eval_fitness` on n = genes.len() / 6 poses.
    pub fn score_poses(&self, genes: &[f64], prec: gd_precision) -> Result<Vec<gd_pose_energy>, Error> {
        let n = genes.len() / 6;
        let mut out = vec![gd_pose_energy::default(); n];
        let st = unsafe { gd_score_poses(self.raw, genes.as_ptr(), n as i32, prec, out.as_mut_ptr()) };
        check(self.ctx, st)?;
        Ok(out)
    }

    /// The `score` command's energies of n models (xyz: n x ligand atoms x 3).
    pub fn score_models(&self, xyz: &[f64], n_models: usize, prec: gd_precision)
                        -> Result<Vec<gd_pose_energy>, Error> {
        let mut out = vec![gd_pose_energy::default(); n_models];
        let st = unsafe { gd_score_models(self.raw, xyz.as_ptr(), n_models as i32, prec, out.as_mut_ptr()) };
        check(self.ctx, st)?;
        Ok(out)
    }

    /// `cluster_structures` of the poses given as genes: (centre, members)
    /// per cluster, in gdock's output order.
    pub fn cluster(&self, genes: &[f64], cfg: &gd_cluster_cfg) -> Result<Vec<(usize, Vec<usize>)>, Error> {
        let n = genes.len() / 6;
        let (mut centers, mut sizes, mut members) = (vec![0i32; n.max(1)], vec![0i32; n.max(1)], vec![0i32; n.max(1)]);
        let mut k = 0i32;
        let st = unsafe {
            gd_cluster(self.raw, genes.as_ptr(), n as i32, cfg, &mut k, centers.as_mut_ptr(), sizes.as_mut_ptr(),
                       members.as_mut_ptr())
        };
        check(self.ctx, st)?;
        Ok(unflatten(k, &centers, &sizes, &members))
    }
}

impl Drop for Complex {
    fn drop(&mut self) {
        unsafe {
            gd_complex_destroy(self.raw);
        }
    }
}

/// (centre, members) per cluster from the flat outputs of `gd_cluster` /
/// `gd_cluster_sets`.
pub fn unflatten(k: i32, centers: &[i32], sizes: &[i32], members: &[i32]) -> Vec<(usize, Vec<usize>)> {
    let mut out = Vec::with_capacity(k.max(0) as usize);
    let mut m = 0usize;
    for c in 0..k.max(0) as usize {
        let s = sizes[c] as usize;
        out.push((centers[c] as usize, members[m..m + s].iter().map(|&v| v as usize).collect()));
        m += s;
    }
    out
}

/// `cluster_structures` on contact sets given as "cA rA cB rB" keys
/// (`gd_pose_contacts`' encoding: (chainA << 48) | (resA << 32) |
/// (chainB << 16) | resB, smaller chain first, ascending per set).
pub fn cluster_sets(ctx: &Context, sets: &[Vec<i64>], cfg: &gd_cluster_cfg) -> Result<Vec<(usize, Vec<usize>)>, Error> {
    let n = sets.len();
    let mut offsets = vec![0i64; n + 1];
    for (i, s) in sets.iter().enumerate() {
        offsets[i + 1] = offsets[i] + s.len() as i64;
    }
    let keys: Vec<i64> = sets.iter().flatten().copied().collect();
    let (mut centers, mut sizes, mut members) = (vec![0i32; n.max(1)], vec![0i32; n.max(1)], vec![0i32; n.max(1)]);
    let mut k = 0i32;
    let st = unsafe {
        gd_cluster_sets(ctx.raw, if keys.is_empty() { std::ptr::null() } else { keys.as_ptr() }, offsets.as_ptr(),
                        n as i32, cfg, &mut k, centers.as_mut_ptr(), sizes.as_mut_ptr(), members.as_mut_ptr())
    };
    check(ctx.raw, st)?;
    Ok(unflatten(k, &centers, &sizes, &members))
}

/// A contact key of `gd_pose_contacts` from the two residues, smaller chain
/// first, as gdock's "cA rA cB rB" strings order them (src/clustering.rs:100-105).
pub fn contact_key(chain_a: char, res_a: i16, chain_b: char, res_b: i16) -> i64 {
    let (ca, ra, cb, rb) = if chain_a > chain_b { (chain_b, res_b, chain_a, res_a) } else { (chain_a, res_a, chain_b, res_b) };
    ((ca as u8 as i64) << 48) | ((ra as u16 as i64) << 32) | ((cb as u8 as i64) << 16) | (rb as u16 as i64)
}

#[cfg(test)]
mod tests {
    use super::*;

    #[test]
    fn names_pack_little_endian() {
        assert_eq!(pack_name(" CA "), u32::from_le_bytes([b'C', b'A', 0, 0]));
        assert_eq!(pack_name("OXT1X"), u32::from_le_bytes([b'O', b'X', b'T', b'1']));
    }

    #[test]
    fn element_classes() {
        assert_eq!(element_class(" C"), GD_ELEM_C);
        assert_eq!(element_class("S"), GD_ELEM_S);
        assert_eq!(element_class("FE"), GD_ELEM_OTHER);
    }

    #[test]
    fn struct_sizes_match_the_header() {
        use std::mem::size_of;
        assert_eq!(size_of::<gd_pose_energy>(), 48);
        assert_eq!(size_of::<gd_pose_frame>(), 128);
        assert_eq!(size_of::<gd_hof_entry>(), 64);
        assert_eq!(size_of::<gd_atoms>(), 8 + 12 * 8);
    }

    #[test]
    fn contact_keys_put_the_smaller_chain_first() {
        assert_eq!(contact_key('B', 7, 'A', 3), contact_key('A', 3, 'B', 7));
    }
}
