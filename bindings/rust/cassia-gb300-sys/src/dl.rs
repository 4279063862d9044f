//! The cassia-format consumer loaded at run time, for callers that load the
//! painter the way the reference demo loads libcassia (a `dlopen` container
//! over `cassia_init / cassia_render / cassia_shutdown`,
//! cassia/src/Cassia.h:32-41).  `cassia_init(w, h)` becomes a composition
//! handle plus a host RGBA8 frame, `cassia_render(segments, stylings)` becomes
//! `cgb_cassia_render` into that frame (headless: the pixels are returned
//! instead of shown), and `cassia_shutdown` becomes `cgb_composition_free`.

use std::os::raw::{c_char, c_void};
use std::ptr;

use dlopen::wrapper::{Container, WrapperApi};
use dlopen_derive::WrapperApi;

use crate::{cgb_buffer, cgb_cassia_styling, cgb_status, CGB_MEMORY_HOST, CGB_OK};

#[derive(WrapperApi)]
struct CassiaGb300Api {
    cgb_composition_new: unsafe extern "C" fn(flags: u32, hbm_budget_bytes: u64, out: *mut *mut c_void) -> cgb_status,
    cgb_composition_free: unsafe extern "C" fn(c: *mut c_void) -> cgb_status,
    cgb_cassia_render: unsafe extern "C" fn(
        c: *mut c_void,
        segments: *const u64,
        n: usize,
        stylings: *const cgb_cassia_styling,
        m: usize,
        buffer: *const cgb_buffer,
        background: *const f32,
    ) -> cgb_status,
    cgb_last_error: unsafe extern "C" fn() -> *const c_char,
}

pub struct CassiaGb300 {
    cont: Container<CassiaGb300Api>,
    handle: *mut c_void,
    width: usize,
    height: usize,
    pixels: Vec<u8>,
    background: [f32; 4],
}

impl CassiaGb300 {
    /// `cassia_init(width, height)`.  `flags` is 0, or
    /// `CGB_COMPOSITION_WIDE_LAYERS` for segments in the widened format.
    pub fn new(lib_path: &str, width: usize, height: usize, flags: u32) -> Result<Self, String> {
        let cont: Container<CassiaGb300Api> =
            unsafe { Container::load(lib_path) }.map_err(|e| format!("{}: {}", lib_path, e))?;
        let mut handle = ptr::null_mut();
        let st = unsafe { cont.cgb_composition_new(flags, 0, &mut handle) };
        if st != CGB_OK {
            return Err(format!("cgb_composition_new: status {}", st));
        }
        Ok(Self { cont, handle, width, height, pixels: vec![0; width * height * 4], background: [1.0; 4] })
    }

    /// The clear colour (linear RGBA) under the painted segments.
    pub fn set_background(&mut self, background: [f32; 4]) {
        self.background = background;
    }

    /// `cassia_render(segments, stylings)`: the reference's `CompactSegment`s
    /// (any order, NONE slots allowed) and one styling per layer order.
    /// Returns the RGBA8 frame, `width * height * 4` bytes.
    pub fn render(&mut self, pixel_segments: &[u64], stylings: &[cgb_cassia_styling]) -> Result<&[u8], String> {
        let buffer = cgb_buffer {
            pixels: self.pixels.as_mut_ptr(),
            width: self.width as u64,
            height: self.height as u64,
            width_stride: 0,
            layer_cache: -1,
            memory: CGB_MEMORY_HOST,
            flusher: None,
            flusher_user: ptr::null_mut(),
        };
        let st = unsafe {
            self.cont.cgb_cassia_render(
                self.handle,
                pixel_segments.as_ptr(),
                pixel_segments.len(),
                stylings.as_ptr(),
                stylings.len(),
                &buffer,
                self.background.as_ptr(),
            )
        };
        if st != CGB_OK {
            let msg = unsafe { std::ffi::CStr::from_ptr(self.cont.cgb_last_error()) };
            return Err(format!("cgb_cassia_render: status {}: {}", st, msg.to_string_lossy()));
        }
        Ok(&self.pixels)
    }
}

impl Drop for CassiaGb300 {
    /// `cassia_shutdown()`.
    fn drop(&mut self) {
        unsafe {
            self.cont.cgb_composition_free(self.handle);
        }
    }
}
