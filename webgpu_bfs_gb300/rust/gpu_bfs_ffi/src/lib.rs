//! Rust binding of `libmsbfs.so`, the GB300 multi-source BFS engine.
//!
//! This is the shim a maintainer adds to the reference workspace (as
//! `crates/gpu_bfs_ffi`) so Rust callers of `GpuBfsEngine`
//! (crates/gpu_bfs/src/engine.rs:57-490) and of the `BfsEngine` trait
//! (crates/core/src/lib.rs:21-39) can run on the CUDA engine instead of the
//! wgpu path. Every function below calls the C ABI of `include/msbfs.h`;
//! no computation happens on the Rust side. With the `reference` feature the
//! engine implements `webgpu_bfs_core::BfsEngine`.
//!
//! Result contract (identical to the reference): `dist[s * V + v]`, `u32`,
//! unreachable = `u32::MAX`, `dist[s * V + sources[s]] == 0`.

use std::ffi::{CStr, CString};
use std::fmt;
use std::os::raw::{c_char, c_int, c_void};

/// Same names and numbering as `GpuBfsMethod` (engine.rs:33-53) and
/// `msbfs_method`.
#[repr(i32)]
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum GpuBfsMethod {
    NaiveSequential = 0,
    BatchedDenseSpMM = 1,
    BitParallel32 = 2,
    BitParallel64 = 3,
    BitParallel64Pull = 4,
    BooleanReachability = 5,
    PushPullAdaptive = 6,
    SparseQueue = 7,
    SparseBitParallel64 = 8,
    MultiWordBitParallel = 9,
    IndirectMacroBatch = 10,
    IndirectSparseQueuePush = 11,
    MultiWordBitParallelPush = 12,
    WorkgroupPersistentBfs = 13,
    Auto = 14,
}

impl GpuBfsMethod {
    fn from_code(code: c_int) -> Option<Self> {
        use GpuBfsMethod::*;
        const ALL: [GpuBfsMethod; 15] = [
            NaiveSequential, BatchedDenseSpMM, BitParallel32, BitParallel64, BitParallel64Pull,
            BooleanReachability, PushPullAdaptive, SparseQueue, SparseBitParallel64,
            MultiWordBitParallel, IndirectMacroBatch, IndirectSparseQueuePush,
            MultiWordBitParallelPush, WorkgroupPersistentBfs, Auto,
        ];
        ALL.get(usize::try_from(code).ok()?).copied()
    }
}

/// `msbfs_stats`: what a call ran and how long it took on the device.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct MsbfsStats {
    pub method: u32,
    pub path: u32,
    pub passes: u32,
    pub words_per_vertex: u32,
    pub levels: u32,
    pub push_levels: u32,
    pub pull_levels: u32,
    pub cta_cluster: u32,
    pub reached_pairs: u64,
    pub gpu_ms: f64,
}

/// `msbfs_tuning`: settings chosen by the level-path autotuner.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct MsbfsTuning {
    pub max_words_per_pass: u32,
    pub alpha: u32,
    pub beta: u32,
    pub hub_split: u32,
    pub bitmap_div: u32,
    pub warp_scan_degree: u32,
    pub from_cache: u32,
    pub trials: u32,
    pub level_path: u32,
    pub ms: f64,
    pub default_ms: f64,
    pub class_name: [c_char; 48],
}

impl Default for MsbfsTuning {
    fn default() -> Self {
        MsbfsTuning {
            max_words_per_pass: 0,
            alpha: 0,
            beta: 0,
            hub_split: 0,
            bitmap_div: 0,
            warp_scan_degree: 0,
            from_cache: 0,
            trials: 0,
            level_path: 0,
            ms: 0.0,
            default_ms: 0.0,
            class_name: [0; 48],
        }
    }
}

#[link(name = "msbfs")]
extern "C" {
    fn msbfs_engine_create(device: c_int, method: c_int, out: *mut *mut c_void) -> c_int;
    fn msbfs_engine_destroy(engine: *mut c_void);
    fn msbfs_engine_method(engine: *const c_void) -> c_int;
    fn msbfs_engine_last_error(engine: *const c_void) -> *const c_char;
    fn msbfs_engine_set_tuning(engine: *mut c_void, max_words: u32, alpha: u32, beta: u32) -> c_int;
    fn msbfs_engine_autotune(engine: *mut c_void, graph: *mut c_void, sources: *const u32,
                             num_sources: usize, cache_path: *const c_char,
                             out: *mut MsbfsTuning) -> c_int;
    fn msbfs_select_auto_method(num_vertices: usize, num_edges: usize, row_offsets: *const u32,
                                num_sources: usize) -> c_int;
    fn msbfs_graph_create(engine: *mut c_void, num_vertices: usize, num_edges: usize,
                          row_offsets: *const u32, col_indices: *const u32,
                          out: *mut *mut c_void) -> c_int;
    fn msbfs_graph_destroy(graph: *mut c_void);
    fn msbfs_run_ms_bfs_with_method(engine: *mut c_void, method: c_int, graph: *const c_void,
                                    sources: *const u32, num_sources: usize, out: *mut u32,
                                    stats: *mut MsbfsStats) -> c_int;
    fn msbfs_run_reachability(engine: *mut c_void, graph: *const c_void, sources: *const u32,
                              num_sources: usize, words: *mut u32,
                              stats: *mut MsbfsStats) -> c_int;
}

/// An error returned by the engine: the `MSBFS_ERR_*` code and the engine's
/// message (the reference's anyhow text where one exists, e.g. "Source
/// vertex 7 at index 2 exceeds graph vertex count 5").
#[derive(Clone, Debug, PartialEq, Eq)]
pub struct MsbfsError {
    pub code: i32,
    pub message: String,
}

impl fmt::Display for MsbfsError {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        write!(f, "{} (msbfs error {})", self.message, self.code)
    }
}

impl std::error::Error for MsbfsError {}

pub type Result<T> = std::result::Result<T, MsbfsError>;

/// A CSR graph borrowed from the caller (`CsrGraph`, crates/core/src/graph.rs:8-22).
#[derive(Clone, Copy, Debug)]
pub struct CsrView<'a> {
    pub num_vertices: usize,
    pub row_offsets: &'a [u32],
    pub col_indices: &'a [u32],
}

/// A graph kept resident in HBM by one engine.
pub struct DeviceGraph {
    handle: *mut c_void,
    num_vertices: usize,
}

impl DeviceGraph {
    pub fn num_vertices(&self) -> usize {
        self.num_vertices
    }
}

impl Drop for DeviceGraph {
    fn drop(&mut self) {
        // SAFETY: the handle came from msbfs_graph_create and is dropped once.
        unsafe { msbfs_graph_destroy(self.handle) }
    }
}

/// `GpuBfsEngine` on the CUDA engine. The library serialises calls on one
/// engine with an internal mutex, so the handle may be shared across threads.
pub struct CudaBfsEngine {
    handle: *mut c_void,
}

// SAFETY: libmsbfs locks a mutex per engine around every call.
unsafe impl Send for CudaBfsEngine {}
unsafe impl Sync for CudaBfsEngine {}

impl CudaBfsEngine {
    /// `GpuBfsEngine::new` (engine.rs:68-78) on CUDA device `device`.
    pub fn new(device: i32, method: GpuBfsMethod) -> Result<Self> {
        let mut handle = std::ptr::null_mut();
        // SAFETY: `handle` is a valid out-pointer.
        let rc = unsafe { msbfs_engine_create(device, method as c_int, &mut handle) };
        if rc != 0 {
            return Err(MsbfsError { code: rc, message: "engine creation failed".into() });
        }
        Ok(CudaBfsEngine { handle })
    }

    /// `GpuBfsEngine::method` (engine.rs:209-212).
    pub fn method(&self) -> GpuBfsMethod {
        // SAFETY: valid engine handle.
        let code = unsafe { msbfs_engine_method(self.handle) };
        GpuBfsMethod::from_code(code).unwrap_or(GpuBfsMethod::Auto)
    }

    /// `GpuBfsEngine::select_auto_method` (engine.rs:157-198).
    pub fn select_auto_method(graph: CsrView<'_>, num_sources: usize) -> GpuBfsMethod {
        let offsets = if graph.num_vertices == 0 { std::ptr::null() } else { graph.row_offsets.as_ptr() };
        // SAFETY: row_offsets holds num_vertices + 1 entries (or none when V == 0).
        let code = unsafe {
            msbfs_select_auto_method(graph.num_vertices, graph.col_indices.len(), offsets,
                                     num_sources)
        };
        GpuBfsMethod::from_code(code).unwrap_or(GpuBfsMethod::Auto)
    }

    fn error(&self, code: c_int) -> MsbfsError {
        // SAFETY: the library returns a NUL-terminated string owned by the engine.
        let message = unsafe {
            let p = msbfs_engine_last_error(self.handle);
            if p.is_null() { String::new() } else { CStr::from_ptr(p).to_string_lossy().into_owned() }
        };
        MsbfsError { code, message }
    }

    /// Uploads a graph (validated like `CsrGraph::validate`) and keeps it
    /// resident; reuse the handle for repeated queries on the same graph.
    pub fn upload(&self, graph: CsrView<'_>) -> Result<DeviceGraph> {
        if graph.row_offsets.len() != graph.num_vertices + 1 {
            return Err(MsbfsError { code: 6, message: "row_offsets must hold V + 1 entries".into() });
        }
        let mut handle = std::ptr::null_mut();
        // SAFETY: the slices outlive the call; the library copies them.
        let rc = unsafe {
            msbfs_graph_create(self.handle, graph.num_vertices, graph.col_indices.len(),
                               graph.row_offsets.as_ptr(), graph.col_indices.as_ptr(), &mut handle)
        };
        if rc != 0 {
            return Err(self.error(rc));
        }
        Ok(DeviceGraph { handle, num_vertices: graph.num_vertices })
    }

    /// `run_ms_bfs_with_method` (engine.rs:300-405) on a resident graph,
    /// into `out` (resized to S * V like `run_ms_bfs_into`, engine.rs:219).
    pub fn run_on_into(&self, method: GpuBfsMethod, graph: &DeviceGraph, sources: &[u32],
                       out: &mut Vec<u32>) -> Result<MsbfsStats> {
        let mut stats = MsbfsStats::default();
        out.clear();
        if sources.is_empty() {
            return Ok(stats);
        }
        if graph.num_vertices == 0 {
            return Err(MsbfsError {
                code: 2,
                message: format!("Source vertex {} at index 0 exceeds graph vertex count 0", sources[0]),
            });
        }
        out.resize(sources.len() * graph.num_vertices, u32::MAX);
        // SAFETY: `out` holds S * V u32; sources holds S entries.
        let rc = unsafe {
            msbfs_run_ms_bfs_with_method(self.handle, method as c_int, graph.handle, sources.as_ptr(),
                                         sources.len(), out.as_mut_ptr(), &mut stats)
        };
        if rc != 0 {
            return Err(self.error(rc));
        }
        Ok(stats)
    }

    /// `GpuBfsEngine::run_ms_bfs_into` (engine.rs:219-298): uploads the
    /// graph for this call.
    pub fn run_ms_bfs_into(&self, graph: CsrView<'_>, sources: &[u32], out: &mut Vec<u32>) -> Result<()> {
        self.run_ms_bfs_with_method_into(self.method(), graph, sources, out)
    }

    /// `GpuBfsEngine::run_ms_bfs_with_method` (engine.rs:300-405).
    pub fn run_ms_bfs_with_method_into(&self, method: GpuBfsMethod, graph: CsrView<'_>,
                                       sources: &[u32], out: &mut Vec<u32>) -> Result<()> {
        if sources.is_empty() {
            out.clear();
            return Ok(());
        }
        let g = self.upload(graph)?;
        self.run_on_into(method, &g, sources, out).map(|_| ())
    }

    /// `BfsEngine::run_ms_bfs` (crates/core/src/lib.rs:38).
    pub fn run_ms_bfs(&self, graph: CsrView<'_>, sources: &[u32]) -> Result<Vec<u32>> {
        let mut out = Vec::new();
        self.run_ms_bfs_into(graph, sources, &mut out)?;
        Ok(out)
    }

    /// `GpuBfsEngine::run_ms_reachability` (engine.rs:420-479): words of
    /// `ReachabilityBitmask` (`words[v * wpv + s / 32]`), with wpv.
    pub fn run_ms_reachability(&self, graph: CsrView<'_>, sources: &[u32]) -> Result<(Vec<u32>, usize)> {
        let wpv = (sources.len() + 31) / 32;
        let mut words = vec![0u32; graph.num_vertices * wpv];
        if sources.is_empty() || graph.num_vertices == 0 {
            return Ok((words, wpv));
        }
        let g = self.upload(graph)?;
        let mut stats = MsbfsStats::default();
        // SAFETY: `words` holds V * ceil(S / 32) u32.
        let rc = unsafe {
            msbfs_run_reachability(self.handle, g.handle, sources.as_ptr(), sources.len(),
                                   words.as_mut_ptr(), &mut stats)
        };
        if rc != 0 {
            return Err(self.error(rc));
        }
        Ok((words, wpv))
    }

    /// Level-path thresholds (no reference counterpart; the reference fixes
    /// alpha = 14, beta = 24 in push_pull.rs:29-36). Zero keeps a value.
    pub fn set_tuning(&self, max_words_per_pass: u32, alpha: u32, beta: u32) -> Result<()> {
        // SAFETY: valid engine handle.
        let rc = unsafe { msbfs_engine_set_tuning(self.handle, max_words_per_pass, alpha, beta) };
        if rc != 0 { Err(self.error(rc)) } else { Ok(()) }
    }

    /// The level-path autotuner (`msbfs_engine_autotune`) for this graph's
    /// class and this source count, with an optional cache file.
    pub fn autotune(&self, graph: &DeviceGraph, sources: &[u32], cache_path: Option<&str>) -> Result<MsbfsTuning> {
        let path = match cache_path {
            Some(p) => Some(CString::new(p).map_err(|_| MsbfsError { code: 7, message: "cache path holds a NUL".into() })?),
            None => None,
        };
        let mut t = MsbfsTuning::default();
        // SAFETY: valid handles; `path` outlives the call.
        let rc = unsafe {
            msbfs_engine_autotune(self.handle, graph.handle, sources.as_ptr(), sources.len(),
                                  path.as_ref().map_or(std::ptr::null(), |c| c.as_ptr()), &mut t)
        };
        if rc != 0 { Err(self.error(rc)) } else { Ok(t) }
    }
}

impl Drop for CudaBfsEngine {
    fn drop(&mut self) {
        // SAFETY: the handle came from msbfs_engine_create and is dropped once.
        unsafe { msbfs_engine_destroy(self.handle) }
    }
}

#[cfg(feature = "reference")]
impl webgpu_bfs_core::BfsEngine for CudaBfsEngine {
    fn run_ms_bfs(&self, graph: &webgpu_bfs_core::CsrGraph, sources: &[u32]) -> anyhow::Result<Vec<u32>> {
        let view = CsrView {
            num_vertices: graph.num_vertices,
            row_offsets: &graph.row_offsets,
            col_indices: &graph.col_indices,
        };
        CudaBfsEngine::run_ms_bfs(self, view, sources).map_err(|e| anyhow::anyhow!(e.message))
    }
}

#[cfg(test)]
mod tests {
    use super::*;

    // The router runs on the host: no GPU needed (engine.rs:502-605 cases).
    #[test]
    fn auto_router_follows_the_reference_branches() {
        // a 4-vertex path: max degree 2, E <= 4V -> workgroup-persistent BFS
        let ro = [0u32, 1, 3, 5, 6];
        let ci = [1u32, 0, 2, 1, 3, 2];
        let g = CsrView { num_vertices: 4, row_offsets: &ro, col_indices: &ci };
        assert_eq!(CudaBfsEngine::select_auto_method(g, 8), GpuBfsMethod::WorkgroupPersistentBfs);
        let empty = CsrView { num_vertices: 0, row_offsets: &[0], col_indices: &[] };
        assert_eq!(CudaBfsEngine::select_auto_method(empty, 8), GpuBfsMethod::NaiveSequential);
    }

    // Needs a CUDA device: `cargo test -- --ignored`.
    #[test]
    #[ignore]
    fn grid_distances_are_manhattan() {
        let (w, h) = (16usize, 16usize);
        let v = w * h;
        let mut ro = vec![0u32];
        let mut ci = Vec::new();
        for y in 0..h {
            for x in 0..w {
                // N, W, E, S neighbour order (generators.rs:28-80)
                if y > 0 { ci.push(((y - 1) * w + x) as u32); }
                if x > 0 { ci.push((y * w + x - 1) as u32); }
                if x + 1 < w { ci.push((y * w + x + 1) as u32); }
                if y + 1 < h { ci.push(((y + 1) * w + x) as u32); }
                ro.push(ci.len() as u32);
            }
        }
        let g = CsrView { num_vertices: v, row_offsets: &ro, col_indices: &ci };
        let eng = CudaBfsEngine::new(0, GpuBfsMethod::Auto).expect("CUDA device");
        let sources = [0u32, 17, 255];
        let dist = eng.run_ms_bfs(g, &sources).expect("run");
        for (s, &src) in sources.iter().enumerate() {
            let (sx, sy) = (src as usize % w, src as usize / w);
            for u in 0..v {
                let (ux, uy) = (u % w, u / w);
                let want = (sx as i64 - ux as i64).abs() + (sy as i64 - uy as i64).abs();
                assert_eq!(dist[s * v + u] as i64, want);
            }
        }
        let err = eng.run_ms_bfs(g, &[3, 4, v as u32]).unwrap_err();
        assert_eq!(err.code, 1);
        assert_eq!(err.message, format!("Source vertex {} at index 2 exceeds graph vertex count {}", v, v));
    }
}
