"""Host mirror of Wflow.jl's model API on the hot path, over the C ABI.

Names follow the reference so that a caller (and the tests) read like Wflow:
  Model(config, domain)            Model(config) for the `sbm` hot-path state (sbm_model.jl:7-57)
  model.update_model()             update_model! + compute_mass_balance! (sbm_model.jl:60-92,
                                   mass_balance.jl:541-545) on the GPU
  model.run_timestep(P, PET, T)    run_timestep! (Wflow.jl:311-322) with the forcing of the step
  model.get_value / set_value      BMI get_value / set_value (bmi.jl:208-248)
  model.save_state / load_state    BMI save_state / load_state (bmi.jl:357-371)
Errors from the library raise RuntimeError with the library's message, like the reference's
throw-and-log behaviour. There is no CPU fallback: without the CUDA library this module fails.
"""

import ctypes as C

import numpy as np

from . import abi, synthetic


class Model:
    def __init__(self, config, domain, params=None, device=0, reservoirs=None):
        self.lib = abi.load_library(required=True)
        self.config = config
        self.domain = domain
        self._params = params if params is not None else domain.params
        self._d, self._p = synthetic.c_structs(domain, self._params)
        h = C.c_void_p()
        if reservoirs is not None:
            # ReservoirModel (reservoir.jl:290-300) at the reservoirs' river cells
            # (with the S-H / H-Q tables and links of the dict's table keys, when it has them)
            self._reservoirs = reservoirs
            self._r = synthetic.c_reservoirs(reservoirs)
            self._rt = synthetic.c_reservoir_tables(reservoirs)
            st = self.lib.wf_create_with_reservoir_tables(
                C.byref(config), C.byref(self._d), C.byref(self._p), C.byref(self._r),
                C.byref(self._rt) if self._rt is not None else None, int(device), C.byref(h))
        else:
            st = self.lib.wf_create(C.byref(config), C.byref(self._d), C.byref(self._p), int(device), C.byref(h))
        if st != abi.WF_OK:
            msg = self.lib.wf_last_error(None)
            raise RuntimeError(f"wf_create failed with status {st}: {msg.decode() if msg else ''}")
        self.h = h
        self.n = domain.n_land
        self.nr = domain.n_river
        self.M = max(1, config.n_members)
        self.N = config.n_soil_layer_thickness + 1
        self.nres = 0 if reservoirs is None else int(reservoirs["river_index"].size)
        self._tune_state = dict(vertical_block=0, routing_warps=0, routing_blocks_per_sm=0)

    def close(self):
        if getattr(self, "h", None):
            self.lib.wf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st != abi.WF_OK:
            msg = self.lib.wf_last_error(self.h)
            raise RuntimeError(f"{what} failed with status {st}: {msg.decode() if msg else ''}")

    # ---- stepping
    def set_forcing(self, precipitation, potential_evaporation, temperature):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (precipitation, potential_evaporation, temperature)]
        cnt = arrs[0].size
        self._check(self.lib.wf_set_forcing(self.h, *[abi.as_ptr(a) for a in arrs], cnt), "wf_set_forcing")

    def set_forcing_async(self, precipitation, potential_evaporation, temperature):
        """wf_set_forcing_async: the copies overlap a step still running. The arrays (pinned
        host memory for a real overlap) are kept referenced until the next step returns."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (precipitation, potential_evaporation, temperature)]
        self._pending_forcing = arrs
        self._check(self.lib.wf_set_forcing_async(self.h, *[abi.as_ptr(a) for a in arrs], arrs[0].size),
                    "wf_set_forcing_async")

    def attach_local_inertial(self, domain):
        """wf_attach_local_inertial: route the land and river by `domain` (a li_river.LiDomain over
        this model's cells) inside every step, in place of the kinematic waves. The model keeps a
        reference to the domain."""
        self._check(self.lib.wf_attach_local_inertial(self.h, domain.h), "wf_attach_local_inertial")
        self._li = domain

    def set_forcing_f32(self, precipitation, potential_evaporation, temperature, asynchronous=False):
        """wf_set_forcing_f32 / wf_set_forcing_async_f32: the forcing as FP32 arrays (half the bytes
        to copy; the split form computes with FP32 forcing anyway)."""
        arrs = [np.ascontiguousarray(a, dtype=np.float32) for a in (precipitation, potential_evaporation, temperature)]
        if asynchronous:
            self._pending_forcing = arrs
        # each array: one set per member, or one set for every member
        f = self.lib.wf_set_forcing_counts_async_f32 if asynchronous else self.lib.wf_set_forcing_counts_f32
        args = [x for a in arrs for x in (abi.as_ptr(a, C.c_float), a.size)]
        self._check(f(self.h, *args), "wf_set_forcing_f32")

    def update_model(self):
        self._check(self.lib.wf_step(self.h), "wf_step")

    def run_timestep(self, precipitation, potential_evaporation, temperature):
        self.set_forcing(precipitation, potential_evaporation, temperature)
        self.update_model()

    def update_model_static(self):
        """The step without any allocation (wf_step_static): scratch from a fixed 16 MiB device
        array shared by all models on the device; calls must not overlap on the GPU."""
        self._check(self.lib.wf_step_static(self.h), "wf_step_static")

    def set_rating_curve_day(self, day_of_year):
        """wf_set_rating_curve_day: the H-Q tables' column the next steps read (col_index_hq =
        julian_day(time - dt), update_index_hq!, reservoir.jl:376-382)."""
        self._check(self.lib.wf_set_rating_curve_day(self.h, int(day_of_year)), "wf_set_rating_curve_day")

    def step_async(self):
        self._check(self.lib.wf_step_async(self.h), "wf_step_async")

    def synchronize(self):
        self._check(self.lib.wf_synchronize(self.h), "wf_synchronize")

    # ---- BMI-like access
    def _extent(self, fid):
        if abi.is_reservoir_field(fid):
            return self.nres
        return self.nr if abi.is_river_field(fid) else self.n

    def get_value(self, field, layer=0, offset=0, count=None):
        fid = abi.FIELD[field] if isinstance(field, str) else int(field)
        total = self._extent(fid) * self.M
        count = total - offset if count is None else count
        out = np.empty(count)
        self._check(self.lib.wf_get_field(self.h, fid, layer, abi.as_ptr(out), offset, count), "wf_get_field")
        return out

    def set_value(self, field, values, layer=0, offset=0):
        fid = abi.FIELD[field] if isinstance(field, str) else int(field)
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._check(self.lib.wf_set_field(self.h, fid, layer, abi.as_ptr(v), offset, v.size), "wf_set_field")

    def outlets(self, which=0):
        n_out = C.c_int64()
        no = C.c_int64()
        self.lib.wf_get_sizes(self.h, None, None, C.byref(no), None, None)
        out = np.empty(max(1, no.value * self.M))
        self._check(self.lib.wf_get_outlets(self.h, which, abi.as_ptr(out), out.size, C.byref(n_out)), "wf_get_outlets")
        return out[: n_out.value].copy()

    def substep_signature(self, kind):
        """Adaptive sub-steps: per member, the sum of the squared sub-step sizes of the last step
        in sweep `kind` (0 subsurface, 1 overland, 2 river)."""
        out = np.empty(self.M)
        self._check(self.lib.wf_get_substep_signature(self.h, int(kind), abi.as_ptr(out), self.M),
                    "wf_get_substep_signature")
        return out

    def save_state(self):
        size = C.c_size_t(0)
        self._check(self.lib.wf_get_state(self.h, None, C.byref(size)), "wf_get_state")
        buf = (C.c_char * size.value)()
        self._check(self.lib.wf_get_state(self.h, buf, C.byref(size)), "wf_get_state")
        return bytes(buf)

    def load_state(self, blob):
        buf = C.create_string_buffer(blob, len(blob))
        self._check(self.lib.wf_set_state(self.h, buf, len(blob)), "wf_set_state")

    def metrics(self):
        m = abi.WfMetrics()
        self._check(self.lib.wf_get_metrics(self.h, C.byref(m)), "wf_get_metrics")
        return {k: getattr(m, k) for k, _ in abi.WfMetrics._fields_}

    def set_tuning(self, vertical_block=0, routing_warps=0, routing_blocks_per_sm=0, use_graph=1,
                   wait_budget_us=0, wait_offset=0, kernel_timing=0, substep_lanes=0, sweep_inputs=0,
                   vertical_blocks_per_sm=0, separate_overland_river=0):
        """Launch shape of the step's kernels (results do not depend on it): threads per block of
        the per-cell kernels, warps per block and blocks per SM of the routing sweeps, the cap of
        the sub-step lanes of their diagonal schedule (0: default), the CUDA graph, and test hooks."""
        t = abi.WfTuning()
        t.vertical_block, t.routing_warps, t.routing_blocks_per_sm, t.use_graph = (
            vertical_block, routing_warps, routing_blocks_per_sm, use_graph)
        t.reserved[0] = wait_budget_us
        t.reserved[1] = wait_offset
        t.reserved[2] = kernel_timing
        t.reserved[3] = substep_lanes
        t.reserved[4] = sweep_inputs  # bit k: sweep k (subsurface, overland, river) keeps its inputs in registers
        t.reserved[5] = vertical_blocks_per_sm  # grid of the split vertical kernel (elements per thread)
        t.reserved[6] = separate_overland_river  # 1: split overland and river sweeps in separate launches
        self._check(self.lib.wf_set_tuning(self.h, C.byref(t)), "wf_set_tuning")

    def stream(self):
        s = C.c_void_p()
        self._check(self.lib.wf_get_stream(self.h, C.byref(s)), "wf_get_stream")
        return s.value

    def kernel_times(self):
        ms = np.zeros(5)
        calls = C.c_int64()
        self._check(self.lib.wf_get_kernel_times(self.h, abi.as_ptr(ms), C.byref(calls)), "wf_get_kernel_times")
        return dict(zip(["vertical", "subsurface", "overland", "river", "balance"], ms.tolist())), calls.value

    def set_forcing_device_slots(self, p_ptr, pet_ptr, t_ptr):
        self._check(self.lib.wf_set_forcing_device_slots(self.h, C.c_void_p(p_ptr), C.c_void_p(pet_ptr),
                                                         C.c_void_p(t_ptr)), "wf_set_forcing_device_slots")

    def slot_order(self):
        ns = C.c_int64()
        self.lib.wf_get_slot_order(self.h, None, 0, C.byref(ns))
        out = np.empty(ns.value, np.int64)
        self._check(self.lib.wf_get_slot_order(self.h, out.ctypes.data_as(C.POINTER(C.c_int64)), out.size,
                                               C.byref(ns)), "wf_get_slot_order")
        return out
