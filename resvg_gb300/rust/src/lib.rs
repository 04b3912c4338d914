//! FFI bindings to `libresvg_gb300`, the GB300 rendering backend for resvg.
//!
//! The raw declarations mirror `include/rgpu_tree.h` and `include/resvg_gpu.h`
//! one to one (`#[repr(C)]` structs, `extern "C"` functions).  The safe layer
//! is what `resvg::render` / `resvg::render_node` need behind a feature:
//! build a [`Tree`] from a `usvg::Tree` (one `add_*` call per usvg node, see
//! the crate's INTEGRATION notes), then [`Tree::render`] onto a host pixmap as
//! resvg's C API does (`crates/c-api/lib.rs:875-893`), or [`Tree::render_node`]
//! with an SVG id (`crates/c-api/lib.rs:908-942`).
#![allow(non_camel_case_types)]

use std::ffi::{CStr, CString};
use std::os::raw::{c_char, c_int, c_void};

// ---------------------------------------------------------------- rgpu_tree.h

#[repr(C)]
#[derive(Clone, Copy, Debug, Default, PartialEq)]
pub struct rgpu_transform {
    pub sx: f32,
    pub ky: f32,
    pub kx: f32,
    pub sy: f32,
    pub tx: f32,
    pub ty: f32,
}

pub const RGPU_MOVE: u8 = 0;
pub const RGPU_LINE: u8 = 1;
pub const RGPU_QUAD: u8 = 2;
pub const RGPU_CUBIC: u8 = 3;
pub const RGPU_CLOSE: u8 = 4;

pub const RGPU_NODE_GROUP: u32 = 0;
pub const RGPU_NODE_PATH: u32 = 1;

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rgpu_stop {
    pub offset: f32,
    pub r: u8,
    pub g: u8,
    pub b: u8,
    pub _pad: u8,
    pub opacity: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rgpu_paint {
    pub kind: u32,
    pub r: u8,
    pub g: u8,
    pub b: u8,
    pub _pad: u8,
    pub x1: f32,
    pub y1: f32,
    pub x2: f32,
    pub y2: f32,
    pub cx: f32,
    pub cy: f32,
    pub r_: f32,
    pub fx: f32,
    pub fy: f32,
    pub fr: f32,
    pub spread: u32,
    pub transform: rgpu_transform,
    pub stop_offset: u32,
    pub stop_count: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rgpu_path {
    pub verb_offset: u32,
    pub verb_count: u32,
    pub point_offset: u32,
    pub point_count: u32,
    pub fill_paint: i32,
    pub fill_opacity: f32,
    pub fill_rule: u32,
    pub stroke_paint: i32,
    pub stroke_opacity: f32,
    pub stroke_width: f32,
    pub miter_limit: f32,
    pub line_cap: u32,
    pub line_join: u32,
    pub dash_offset: u32,
    pub dash_count: u32,
    pub dash_phase: f32,
    pub stroke_first: u32,
    pub anti_alias: u32,
    pub visible: u32,
    pub bbox_x: f32,
    pub bbox_y: f32,
    pub bbox_w: f32,
    pub bbox_h: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rgpu_node {
    pub kind: u32,
    pub index: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rgpu_group {
    pub transform: rgpu_transform,
    pub opacity: f32,
    pub blend: u32,
    pub isolate: u32,
    pub clip_path: i32,
    pub mask: i32,
    pub filter_offset: u32,
    pub filter_count: u32,
    pub child_offset: u32,
    pub child_count: u32,
    pub has_layer_bbox: u32,
    pub layer_x: f32,
    pub layer_y: f32,
    pub layer_w: f32,
    pub layer_h: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rgpu_clip {
    pub transform: rgpu_transform,
    pub clip_path: i32,
    pub root: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rgpu_mask {
    pub x: f32,
    pub y: f32,
    pub w: f32,
    pub h: f32,
    pub kind: u32,
    pub mask: i32,
    pub root: u32,
}

pub const RGPU_PRIM_F: usize = 64;

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct rgpu_primitive {
    pub kind: u32,
    pub x: f32,
    pub y: f32,
    pub w: f32,
    pub h: f32,
    pub linear_rgb: u32,
    pub in1: i32,
    pub in2: i32,
    pub i: [i32; 8],
    pub f: [f32; RGPU_PRIM_F],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rgpu_filter {
    pub x: f32,
    pub y: f32,
    pub w: f32,
    pub h: f32,
    pub prim_offset: u32,
    pub prim_count: u32,
}

/// Opaque: the library's resolved tree (the `usvg::Tree` stand-in).
#[repr(C)]
pub struct rgpu_tree {
    _private: [u8; 0],
}
pub type resvg_render_tree = rgpu_tree;

// ---------------------------------------------------------------- resvg_gpu.h

pub const RGPU_OK: c_int = 0;
pub const RGPU_ERR_INVALID_ARG: c_int = 1;
pub const RGPU_ERR_NO_DEVICE: c_int = 2;
pub const RGPU_ERR_CUDA: c_int = 3;
pub const RGPU_ERR_OUT_OF_MEMORY: c_int = 4;
pub const RGPU_ERR_CAPACITY: c_int = 5;
pub const RGPU_ERR_DEVICE_FAULT: c_int = 6;
pub const RGPU_ERR_UNSUPPORTED: c_int = 7;

/// `resvg_transform` of resvg's C API (crates/c-api/lib.rs:67-81).
#[repr(C)]
#[derive(Clone, Copy, Debug, PartialEq)]
pub struct resvg_transform {
    pub a: f32,
    pub b: f32,
    pub c: f32,
    pub d: f32,
    pub e: f32,
    pub f: f32,
}

impl Default for resvg_transform {
    fn default() -> Self {
        resvg_transform { a: 1.0, b: 0.0, c: 0.0, d: 1.0, e: 0.0, f: 0.0 }
    }
}

#[repr(C)]
pub struct rgpu_scene {
    _private: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rgpu_tuning {
    pub band_rows: u32,
    pub pixels_per_thread: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rgpu_stats {
    pub draws: u64,
    pub edges: u64,
    pub crossings_capacity: u64,
    pub work_items: u64,
    pub kernel_launches: u64,
    pub h2d_bytes: u64,
    pub d2h_bytes: u64,
    pub raster_ms: f32,
    pub stroke_ms: f32,
    pub stroke_jobs: u64,
}

/// One path for `rgpu_stroke_paths` (tiny-skia-path's `Path::stroke`).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct rgpu_stroke_desc {
    pub verb_off: u32,
    pub verb_cnt: u32,
    pub pt_off: u32,
    pub pt_cnt: u32,
    pub width: f32,
    pub miter_limit: f32,
    pub res_scale: f32,
    pub cap: u32,
    pub join: u32,
    pub dash_off: u32,
    pub dash_cnt: u32,
    pub dash_phase: f32,
}

#[link(name = "resvg_gb300")]
extern "C" {
    // tree building
    pub fn rgpu_tree_new(width: f32, height: f32) -> *mut resvg_render_tree;
    pub fn rgpu_tree_free(tree: *mut resvg_render_tree);
    pub fn rgpu_tree_add_group(tree: *mut resvg_render_tree, parent: i32, group: *const rgpu_group) -> i32;
    pub fn rgpu_tree_add_path(
        tree: *mut resvg_render_tree,
        parent: i32,
        path: *const rgpu_path,
        verbs: *const u8,
        verb_count: u32,
        points: *const f32,
        point_count: u32,
        dashes: *const f32,
        dash_count: u32,
    ) -> i32;
    pub fn rgpu_tree_add_paint(
        tree: *mut resvg_render_tree,
        paint: *const rgpu_paint,
        stops: *const rgpu_stop,
        stop_count: u32,
    ) -> i32;
    pub fn rgpu_tree_add_clip(tree: *mut resvg_render_tree, clip: *const rgpu_clip) -> i32;
    pub fn rgpu_tree_add_mask(tree: *mut resvg_render_tree, mask: *const rgpu_mask) -> i32;
    pub fn rgpu_tree_add_filter(
        tree: *mut resvg_render_tree,
        filter: *const rgpu_filter,
        prims: *const rgpu_primitive,
        prim_count: u32,
        merge_inputs: *const i32,
        merge_count: u32,
    ) -> i32;
    pub fn rgpu_tree_add_image(tree: *mut resvg_render_tree, width: u32, height: u32, rgba: *const u8) -> i32;
    pub fn rgpu_tree_set_node_id(tree: *mut resvg_render_tree, node_kind: u32, index: u32, id: *const c_char) -> c_int;
    pub fn rgpu_tree_find_node(
        tree: *const resvg_render_tree,
        id: *const c_char,
        node_kind: *mut u32,
        index: *mut u32,
    ) -> c_int;
    pub fn rgpu_tree_set_group_filters(
        tree: *mut resvg_render_tree,
        group: i32,
        filters: *const u32,
        count: u32,
    ) -> c_int;
    pub fn rgpu_tree_finalize(tree: *mut resvg_render_tree) -> c_int;

    // drop-in render
    pub fn resvg_render(
        tree: *const resvg_render_tree,
        transform: resvg_transform,
        width: u32,
        height: u32,
        pixmap: *mut c_char,
    );
    pub fn resvg_render_node(
        tree: *const resvg_render_tree,
        id: *const c_char,
        transform: resvg_transform,
        width: u32,
        height: u32,
        pixmap: *mut c_char,
    ) -> bool;

    // GPU-native entry points
    pub fn rgpu_init(device: c_int) -> c_int;
    pub fn rgpu_last_error() -> *const c_char;
    pub fn rgpu_last_warning() -> *const c_char;
    pub fn rgpu_render_device(
        tree: *const resvg_render_tree,
        transform: resvg_transform,
        width: u32,
        height: u32,
        device_pixmap: *mut u8,
        stride: u32,
        stream: *mut c_void,
    ) -> c_int;
    pub fn rgpu_render_batch(
        trees: *const *const resvg_render_tree,
        transforms: *const resvg_transform,
        count: u32,
        widths: *const u32,
        heights: *const u32,
        device_pixmaps: *const *mut u8,
        stream: *mut c_void,
    ) -> c_int;
    pub fn rgpu_scene_prepare(
        trees: *const *const resvg_render_tree,
        transforms: *const resvg_transform,
        count: u32,
        widths: *const u32,
        heights: *const u32,
        device_pixmaps: *const *mut u8,
        strides: *const u32,
        out: *mut *mut rgpu_scene,
    ) -> c_int;
    pub fn rgpu_scene_render(scene: *mut rgpu_scene, stream: *mut c_void) -> c_int;
    pub fn rgpu_scene_check(scene: *mut rgpu_scene, raster_ms: *mut f32) -> c_int;
    pub fn rgpu_scene_free(scene: *mut rgpu_scene);
    pub fn rgpu_set_tuning(t: *const rgpu_tuning) -> c_int;
    pub fn rgpu_get_tuning(t: *mut rgpu_tuning) -> c_int;
    pub fn rgpu_get_stats(s: *mut rgpu_stats) -> c_int;
    pub fn rgpu_set_wait_limit(rounds: u32) -> c_int;
    pub fn rgpu_trim() -> c_int;
    pub fn rgpu_set_stroke_mode(on_device: c_int) -> c_int;
    pub fn rgpu_stroke_paths(
        descs: *const rgpu_stroke_desc,
        count: u32,
        verbs: *const u8,
        verb_count: u32,
        pts: *const f32,
        pt_count: u32,
        dashes: *const f32,
        dash_count: u32,
        on_device: c_int,
        out_verbs: *mut u8,
        verb_cap: u32,
        out_pts: *mut f32,
        pt_cap: u32,
        out_counts: *mut u32,
    ) -> c_int;
}

// ---------------------------------------------------------------- safe layer

/// An error of the backend: its status and `rgpu_last_error()` text.
#[derive(Debug, Clone)]
pub struct Error {
    pub status: c_int,
    pub message: String,
}

fn last_error() -> String {
    unsafe {
        let p = rgpu_last_error();
        if p.is_null() {
            String::new()
        } else {
            CStr::from_ptr(p).to_string_lossy().into_owned()
        }
    }
}

/// Warnings of this thread's last call (what resvg logs and skips, such as a
/// filter that fails and clears its layer); empty when none.
pub fn last_warning() -> String {
    unsafe {
        let p = rgpu_last_warning();
        if p.is_null() {
            String::new()
        } else {
            CStr::from_ptr(p).to_string_lossy().into_owned()
        }
    }
}

fn check(status: c_int) -> Result<(), Error> {
    if status == RGPU_OK {
        Ok(())
    } else {
        Err(Error { status, message: last_error() })
    }
}

/// An owned tree of the backend, freed on drop.
pub struct Tree {
    raw: *mut resvg_render_tree,
}

impl Tree {
    /// An empty tree of the given canvas size; `None` for a non-positive size.
    pub fn new(width: f32, height: f32) -> Option<Tree> {
        let raw = unsafe { rgpu_tree_new(width, height) };
        if raw.is_null() {
            None
        } else {
            Some(Tree { raw })
        }
    }

    pub fn as_ptr(&self) -> *mut resvg_render_tree {
        self.raw
    }

    pub fn add_group(&mut self, parent: i32, group: &rgpu_group) -> i32 {
        unsafe { rgpu_tree_add_group(self.raw, parent, group) }
    }

    pub fn add_paint(&mut self, paint: &rgpu_paint, stops: &[rgpu_stop]) -> i32 {
        unsafe { rgpu_tree_add_paint(self.raw, paint, stops.as_ptr(), stops.len() as u32) }
    }

    /// `points` are (x, y) pairs; `dashes` the resolved dash array (may be empty).
    pub fn add_path(&mut self, parent: i32, path: &rgpu_path, verbs: &[u8], points: &[f32], dashes: &[f32]) -> i32 {
        unsafe {
            rgpu_tree_add_path(
                self.raw,
                parent,
                path,
                verbs.as_ptr(),
                verbs.len() as u32,
                points.as_ptr(),
                (points.len() / 2) as u32,
                if dashes.is_empty() { std::ptr::null() } else { dashes.as_ptr() },
                dashes.len() as u32,
            )
        }
    }

    /// Gives a node its SVG id (usvg's `Node::id`), for `render_node`.
    pub fn set_node_id(&mut self, kind: u32, index: u32, id: &str) -> Result<(), Error> {
        let c = CString::new(id).map_err(|_| Error { status: RGPU_ERR_INVALID_ARG, message: "id with a NUL".into() })?;
        check(unsafe { rgpu_tree_set_node_id(self.raw, kind, index, c.as_ptr()) })
    }

    pub fn finalize(&mut self) -> Result<(), Error> {
        check(unsafe { rgpu_tree_finalize(self.raw) })
    }

    /// `resvg::render` onto a host pixmap of premultiplied RGBA8,
    /// `width * height * 4` bytes, drawn onto its content.
    pub fn render(&self, transform: resvg_transform, width: u32, height: u32, pixmap: &mut [u8]) -> Result<(), Error> {
        if pixmap.len() != width as usize * height as usize * 4 {
            return Err(Error { status: RGPU_ERR_INVALID_ARG, message: "pixmap size".into() });
        }
        unsafe { resvg_render(self.raw, transform, width, height, pixmap.as_mut_ptr() as *mut c_char) };
        let msg = last_error();
        if msg.is_empty() {
            Ok(())
        } else {
            Err(Error { status: RGPU_ERR_CUDA, message: msg })
        }
    }

    /// `resvg::render_node` of the node with SVG id `id`: `Ok(false)` when the
    /// id is unknown or the node's bounding box is empty, as the C API.
    pub fn render_node(
        &self,
        id: &str,
        transform: resvg_transform,
        width: u32,
        height: u32,
        pixmap: &mut [u8],
    ) -> Result<bool, Error> {
        if pixmap.len() != width as usize * height as usize * 4 {
            return Err(Error { status: RGPU_ERR_INVALID_ARG, message: "pixmap size".into() });
        }
        let c = CString::new(id).map_err(|_| Error { status: RGPU_ERR_INVALID_ARG, message: "id with a NUL".into() })?;
        Ok(unsafe { resvg_render_node(self.raw, c.as_ptr(), transform, width, height, pixmap.as_mut_ptr() as *mut c_char) })
    }
}

impl Drop for Tree {
    fn drop(&mut self) {
        unsafe { rgpu_tree_free(self.raw) };
    }
}

/// Selects the CUDA device (the library uses device 0).
pub fn init() -> Result<(), Error> {
    check(unsafe { rgpu_init(0) })
}
