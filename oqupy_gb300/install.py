"""Hook the GPU backends into an imported ``oqupy`` package.

``oqupy.Tempo`` builds its backend as ``TempoBackend(..., config=
backend_config)`` (oqupy/tempo.py:424-435) and ``oqupy.PtTempo`` builds
``PtTempoBackend(..., config=...)`` (oqupy/pt_tempo.py:218-228); both names
are module globals.  ``install()`` rebinds them to factories that return the
GPU backend when ``backend_config["backend"] == "gb300"`` and the reference
class otherwise, so existing code selects the GPU path through its existing
configuration.  The factory dispatches before the reference constructor runs,
so the reference never sees the unknown backend name.

``oqupy.MeanFieldTempo`` builds ``MeanFieldTempoBackend(..., config=...)``
(oqupy/tempo.py:818-832), rebound the same way to ``mean_field.py``'s
batched backend.

``PtTempo.get_process_tensor`` (oqupy/pt_tempo.py:280-306) returns, for a
GPU build, a ``DeviceProcessTensor`` (``device_pt.py``): a
``BaseProcessTensor`` whose tensors stay in device memory.

``compute_dynamics`` has no configuration argument
(oqupy/system_dynamics.py:41-53): the wrapper routes a call to the GPU sweep
when its single process tensor is a ``DeviceProcessTensor``, the system is a
``System`` or ``TimeDependentSystem`` and ``record_all`` is set (control
operations are folded into the sweep's propagators, ``correlations.py``),
and otherwise calls the reference function (a ``DeviceProcessTensor`` that the reference must handle is
first copied to a host ``SimpleProcessTensor``).  Both
``oqupy.system_dynamics.compute_dynamics`` and ``oqupy.compute_dynamics``
(bound at import, oqupy/__init__.py:104) are rebound, and so is
``compute_correlations_nt`` (which ``compute_correlations`` calls): on a
device process tensor its runs become the slots of one batched sweep; and
``oqupy.gradient.compute_gradient_and_dynamics`` (which ``state_gradient``
calls), whose forward and adjoint sweeps run on the GPU; and
``compute_dynamics_with_field`` (mean-field dynamics on process tensors),
whose sweeps advance on the GPU one step per host field update.
"""

from typing import Any, Dict, Optional

import numpy as np

BACKEND_NAME = "gb300"
_installed: Dict[str, Any] = {}


def _wants_gpu(config: Optional[dict]) -> bool:
    return isinstance(config, dict) and config.get("backend") == BACKEND_NAME


def install(oqupy_module: Any = None) -> None:
    """Rebind the backend constructors of ``oqupy`` (idempotent)."""
    if oqupy_module is None:
        import oqupy as oqupy_module  # noqa: F401
    import importlib
    tempo_mod = importlib.import_module(oqupy_module.__name__ + ".tempo")
    from .tempo import GpuTempoBackend

    if "TempoBackend" not in _installed:
        ref_cls = tempo_mod.TempoBackend
        _installed["TempoBackend"] = ref_cls

        def tempo_backend(*args, config=None, degeneracy_maps=None, **kwargs):
            if _wants_gpu(config) and degeneracy_maps is None:
                return GpuTempoBackend(*args, config=config, degeneracy_maps=None, **kwargs)
            if _wants_gpu(config):
                config = {k: v for k, v in config.items() if k != "backend"}
            return ref_cls(*args, config=config, degeneracy_maps=degeneracy_maps, **kwargs)

        tempo_backend.reference_class = ref_cls
        tempo_mod.TempoBackend = tempo_backend

    if "MeanFieldTempoBackend" not in _installed:
        # oqupy.MeanFieldTempo builds MeanFieldTempoBackend(..., config=...,
        # degeneracy_maps_list=...) (oqupy/tempo.py:818-832)
        from .mean_field import GpuMeanFieldTempoBackend
        ref_mf = tempo_mod.MeanFieldTempoBackend
        _installed["MeanFieldTempoBackend"] = ref_mf

        def mean_field_backend(*args, config=None, degeneracy_maps_list=None, **kwargs):
            plain = degeneracy_maps_list is None or all(m is None for m in degeneracy_maps_list)
            if _wants_gpu(config) and plain:
                return GpuMeanFieldTempoBackend(*args, config=config,
                                                degeneracy_maps_list=None, **kwargs)
            if _wants_gpu(config):
                config = {k: v for k, v in config.items() if k != "backend"}
            return ref_mf(*args, config=config, degeneracy_maps_list=degeneracy_maps_list, **kwargs)

        mean_field_backend.reference_class = ref_mf
        tempo_mod.MeanFieldTempoBackend = mean_field_backend

    pt_mod = importlib.import_module(oqupy_module.__name__ + ".pt_tempo")
    from .pt import GpuPtTempoBackend
    if "PtTempoBackend" not in _installed:
        ref_pt = pt_mod.PtTempoBackend
        _installed["PtTempoBackend"] = ref_pt

        def pt_tempo_backend(*args, config=None, degeneracy_maps=None, **kwargs):
            if _wants_gpu(config) and degeneracy_maps is None:
                return GpuPtTempoBackend(*args, config=config, degeneracy_maps=None, **kwargs)
            if _wants_gpu(config):
                config = {k: v for k, v in config.items() if k != "backend"}
            return ref_pt(*args, config=config, degeneracy_maps=degeneracy_maps, **kwargs)

        pt_tempo_backend.reference_class = ref_pt
        pt_mod.PtTempoBackend = pt_tempo_backend

    if "get_process_tensor" not in _installed:
        ref_get = pt_mod.PtTempo.get_process_tensor
        _installed["get_process_tensor"] = ref_get
        ptm = importlib.import_module(oqupy_module.__name__ + ".process_tensor")

        def get_process_tensor(self, progress_type=None):
            be = self._backend_instance
            if not isinstance(be, GpuPtTempoBackend):
                return ref_get(self, progress_type=progress_type)
            if be.step is None or be.step < be.num_steps:
                self.compute(progress_type=progress_type)
            return be.device_process_tensor(ptm.BaseProcessTensor)

        get_process_tensor.reference_function = ref_get
        pt_mod.PtTempo.get_process_tensor = get_process_tensor

    sd_mod = importlib.import_module(oqupy_module.__name__ + ".system_dynamics")
    if "compute_dynamics" not in _installed:
        ref_cd = sd_mod.compute_dynamics
        _installed["compute_dynamics"] = ref_cd
        _installed["compute_dynamics_pkg"] = getattr(oqupy_module, "compute_dynamics", None)
        sys_mod = importlib.import_module(oqupy_module.__name__ + ".system")
        dyn_mod = importlib.import_module(oqupy_module.__name__ + ".dynamics")
        ptm = importlib.import_module(oqupy_module.__name__ + ".process_tensor")
        from .device_pt import device_process_tensor_class
        dev_cls = device_process_tensor_class(ptm.BaseProcessTensor)

        def host_copy(pt):
            return pt.to_host(ptm.SimpleProcessTensor) if isinstance(pt, dev_cls) else pt

        gpu_systems = (sys_mod.System, sys_mod.TimeDependentSystem)

        def compute_dynamics(system, initial_state=None, dt=None, num_steps=None,
                             start_time=0.0, process_tensor=None, control=None,
                             record_all=True, subdiv_limit=None,
                             liouvillian_epsrel=None, progress_type=None):
            kwargs = dict(initial_state=initial_state, dt=dt, num_steps=num_steps,
                          start_time=start_time, process_tensor=process_tensor,
                          control=control, record_all=record_all,
                          progress_type=progress_type)
            if subdiv_limit is not None:
                kwargs["subdiv_limit"] = subdiv_limit
            if liouvillian_epsrel is not None:
                kwargs["liouvillian_epsrel"] = liouvillian_epsrel
            pts = process_tensor if isinstance(process_tensor, list) else \
                ([] if process_tensor is None else [process_tensor])
            gpu = (len(pts) == 1 and isinstance(pts[0], dev_cls) and record_all
                   and type(system) in gpu_systems)
            if not gpu:
                if any(isinstance(p, dev_cls) for p in pts):
                    hosts = [host_copy(p) for p in pts]
                    kwargs["process_tensor"] = hosts if isinstance(process_tensor, list) else hosts[0]
                return ref_cd(system, **kwargs)
            parsed = sd_mod._compute_dynamics_input_parse(
                False, system, initial_state, dt, num_steps, start_time,
                process_tensor, control, record_all)
            system, initial_state, dt, num_steps, start_time = parsed[:5]
            hs_dim = parsed[-1]
            args = [dt, start_time]
            args.append(kwargs.get("subdiv_limit", sd_mod.SUBDIV_LIMIT))
            args.append(kwargs.get("liouvillian_epsrel", sd_mod.INTEGRATE_EPSREL))
            props = system.get_propagators(*args)
            if type(system) is sys_mod.System:
                p1, p2 = props(0)

                def props(step, pair=(p1, p2)):
                    return pair
            ctl = None
            if control is not None:
                # Control.get_controls per step (control.py:119-180), as the
                # reference's loop asks for them (system_dynamics.py:109-114)
                ctl = {"pre": {}, "post": {}}
                for step in range(num_steps + 1):
                    pre, post = control.get_controls(step, dt=dt, start_time=start_time)
                    if pre is not None:
                        ctl["pre"][step] = pre
                    if post is not None:
                        ctl["post"][step] = post
            from . import correlations as corr
            st = corr.device_dynamics(pts[0], [props], [initial_state.reshape(-1)],
                                      num_steps, [ctl])
            states = [s.reshape(hs_dim, hs_dim) for s in st[:, 0]]
            times = start_time + np.arange(len(states)) * dt
            return dyn_mod.Dynamics(times=list(times), states=states)

        compute_dynamics.reference_function = ref_cd
        sd_mod.compute_dynamics = compute_dynamics
        if _installed["compute_dynamics_pkg"] is not None:
            oqupy_module.compute_dynamics = compute_dynamics

        # compute_correlations_nt (system_dynamics.py:791-990; also reached
        # through compute_correlations, :1011-1093): on a device process
        # tensor, every compute_dynamics run of its schedule becomes one slot
        # of a single batched sweep
        ref_nt = sd_mod.compute_correlations_nt
        _installed["compute_correlations_nt"] = ref_nt
        _installed["compute_correlations_nt_pkg"] = getattr(oqupy_module, "compute_correlations_nt", None)

        def compute_correlations_nt(system, process_tensor, operators, ops_times, ops_order,
                                    initial_state=None, start_time=0.0, dt=None,
                                    progress_type=None):
            if not (isinstance(process_tensor, dev_cls) and type(system) in gpu_systems
                    and initial_state is not None):
                if isinstance(process_tensor, dev_cls):
                    process_tensor = host_copy(process_tensor)
                return ref_nt(system, process_tensor, operators, ops_times, ops_order,
                              initial_state=initial_state, start_time=start_time, dt=dt,
                              progress_type=progress_type)
            # the reference's input checks and time parsing (:847-901)
            dim = system.dimension
            assert process_tensor.hilbert_space_dimension == dim
            for op in operators:
                assert np.asarray(op).shape == (dim, dim)
            assert isinstance(start_time, float)
            if dt is None:
                assert process_tensor.dt is not None, \
                    "It is necessary to specify time step `dt` because the given tensor has none."
                dt_ = process_tensor.dt
            else:
                dt_ = dt
            assert len(operators) == len(ops_times) == len(ops_order), \
                "Lengths of the lists ops_order, ops_times and dip_ops do not match."
            max_step = len(process_tensor)
            steps = [sd_mod._parse_times(t, max_step, dt_, start_time) for t in ops_times]
            ret_times = [start_time + dt_ * s for s in steps]
            props = system.get_propagators(dt_, start_time, sd_mod.SUBDIV_LIMIT,
                                           sd_mod.INTEGRATE_EPSREL)
            if type(system) is sys_mod.System:
                p1, p2 = props(0)

                def props(step, pair=(p1, p2)):
                    return pair
            from . import correlations as corr
            rho0 = np.asarray(initial_state, dtype=np.complex128).reshape(-1)
            return ret_times, corr.device_correlations_nt(process_tensor, props, rho0,
                                                          operators, steps, ops_order)

        compute_correlations_nt.reference_function = ref_nt
        sd_mod.compute_correlations_nt = compute_correlations_nt
        if _installed["compute_correlations_nt_pkg"] is not None:
            oqupy_module.compute_correlations_nt = compute_correlations_nt

        # compute_gradient_and_dynamics (oqupy/gradient.py:169-437; reached
        # through state_gradient): on one device process tensor, the forward
        # and adjoint sweeps run on the GPU
        grad_mod = importlib.import_module(oqupy_module.__name__ + ".gradient")
        ref_grad = grad_mod.compute_gradient_and_dynamics
        _installed["compute_gradient_and_dynamics"] = ref_grad

        def compute_gradient_and_dynamics(system, initial_state, target_derivative, process_tensors,
                                          parameters, start_time=0.0, dt=None, num_steps=None,
                                          control=None, record_all=True, progress_type=None):
            pts = process_tensors if isinstance(process_tensors, list) else [process_tensors]
            if not (len(pts) == 1 and isinstance(pts[0], dev_cls) and record_all):
                hosts = [host_copy(p) for p in pts]
                return ref_grad(system, initial_state, target_derivative,
                                hosts if isinstance(process_tensors, list) else hosts[0], parameters,
                                start_time=start_time, dt=dt, num_steps=num_steps, control=control,
                                record_all=record_all, progress_type=progress_type)
            parsed = sd_mod._compute_dynamics_input_parse(
                False, system, initial_state, dt, num_steps, start_time,
                process_tensors, control, record_all)
            system, initial_state, dt, num_steps, start_time = parsed[:5]
            hs_dim = parsed[-1]
            props = system.get_propagators(dt, parameters)
            ctl = None
            if control is not None:
                ctl = {"pre": {}, "post": {}}
                for step in range(num_steps + 1):
                    pre, post = control.get_controls(step, dt=dt, start_time=start_time)
                    if pre is not None:
                        ctl["pre"][step] = pre
                    if post is not None:
                        ctl["post"][step] = post
            from . import correlations as corr
            rho0 = initial_state.reshape(-1)
            target = target_derivative
            if callable(target):
                # the reference evaluates it on the final state (gradient.py:350-351)
                st = corr.device_dynamics(pts[0], [props], [rho0], num_steps, [ctl])
                target = target(st[-1, 0].reshape(hs_dim, hs_dim))
            derivs, states = corr.device_gradient(pts[0], props, rho0, np.asarray(target).reshape(-1),
                                                  num_steps, ctl)
            mats = [s.reshape(hs_dim, hs_dim) for s in states]
            times = start_time + np.arange(len(mats)) * dt
            return list(derivs), dyn_mod.Dynamics(times=list(times), states=mats)

        compute_gradient_and_dynamics.reference_function = ref_grad
        grad_mod.compute_gradient_and_dynamics = compute_gradient_and_dynamics

        # compute_dynamics_with_field (system_dynamics.py:184-476): mean-field
        # dynamics on device process tensors, one sweep step per call
        ref_wf = sd_mod.compute_dynamics_with_field
        _installed["compute_dynamics_with_field"] = ref_wf
        _installed["compute_dynamics_with_field_pkg"] = getattr(oqupy_module, "compute_dynamics_with_field", None)

        def single_device_pt(p):
            if isinstance(p, list):
                return p[0] if len(p) == 1 and isinstance(p[0], dev_cls) else None
            return p if isinstance(p, dev_cls) else None

        def compute_dynamics_with_field(mean_field_system, initial_field, process_tensor_list=None,
                                        dt=None, num_steps=None, initial_state_list=None,
                                        start_time=0.0, control_list=None, record_all=True,
                                        subdiv_limit=sd_mod.SUBDIV_LIMIT,
                                        liouvillian_epsrel=sd_mod.INTEGRATE_EPSREL, progress_type=None):
            kwargs = dict(process_tensor_list=process_tensor_list, dt=dt, num_steps=num_steps,
                          initial_state_list=initial_state_list, start_time=start_time,
                          control_list=control_list, record_all=record_all, subdiv_limit=subdiv_limit,
                          liouvillian_epsrel=liouvillian_epsrel, progress_type=progress_type)
            devs = [single_device_pt(p) for p in (process_tensor_list or [])]
            n_sys = len(mean_field_system.system_list)
            if not (record_all and len(devs) == n_sys and all(d is not None for d in devs)):
                if process_tensor_list is not None:
                    kwargs["process_tensor_list"] = [
                        [host_copy(q) for q in p] if isinstance(p, list) else host_copy(p)
                        for p in process_tensor_list]
                return ref_wf(mean_field_system, initial_field, **kwargs)
            states0 = initial_state_list if initial_state_list is not None else [None] * n_sys
            controls_in = control_list if control_list is not None else [None] * n_sys
            parsed = [sd_mod._compute_dynamics_input_parse(True, system, st, dt, num_steps, start_time,
                                                           pt, ctl, record_all)
                      for system, st, pt, ctl in zip(mean_field_system.system_list, states0,
                                                     process_tensor_list, controls_in)]
            num_steps_, dt_ = parsed[0][3], parsed[0][2]
            props = [system.get_propagators(dt_, start_time, subdiv_limit, liouvillian_epsrel)
                     for system in mean_field_system.system_list]
            ctls = []
            for ctl in controls_in:
                if ctl is None:
                    ctls.append(None)
                    continue
                c = {"pre": {}, "post": {}}
                for step in range(num_steps_ + 1):
                    pre, post = ctl.get_controls(step, dt=dt_, start_time=start_time)
                    if pre is not None:
                        c["pre"][step] = pre
                    if post is not None:
                        c["post"][step] = post
                ctls.append(c)
            from .mean_field import device_dynamics_with_field
            times, states, fields = device_dynamics_with_field(
                props, mean_field_system.field_eom, initial_field, devs,
                [p[1].reshape(-1) for p in parsed], num_steps_, dt_, start_time, ctls)
            return dyn_mod.MeanFieldDynamics(times=times, system_states_list=states, fields=fields)

        compute_dynamics_with_field.reference_function = ref_wf
        sd_mod.compute_dynamics_with_field = compute_dynamics_with_field
        if _installed["compute_dynamics_with_field_pkg"] is not None:
            oqupy_module.compute_dynamics_with_field = compute_dynamics_with_field


def uninstall(oqupy_module: Any = None) -> None:
    if oqupy_module is None:
        import oqupy as oqupy_module  # noqa: F401
    import importlib
    tempo_mod = importlib.import_module(oqupy_module.__name__ + ".tempo")
    if "TempoBackend" in _installed:
        tempo_mod.TempoBackend = _installed.pop("TempoBackend")
    if "MeanFieldTempoBackend" in _installed:
        tempo_mod.MeanFieldTempoBackend = _installed.pop("MeanFieldTempoBackend")
    pt_mod = importlib.import_module(oqupy_module.__name__ + ".pt_tempo")
    if "PtTempoBackend" in _installed:
        pt_mod.PtTempoBackend = _installed.pop("PtTempoBackend")
    if "get_process_tensor" in _installed:
        pt_mod.PtTempo.get_process_tensor = _installed.pop("get_process_tensor")
    if "compute_dynamics" in _installed:
        sd_mod = importlib.import_module(oqupy_module.__name__ + ".system_dynamics")
        sd_mod.compute_dynamics = _installed.pop("compute_dynamics")
        pkg = _installed.pop("compute_dynamics_pkg", None)
        if pkg is not None:
            oqupy_module.compute_dynamics = pkg
        sd_mod.compute_correlations_nt = _installed.pop("compute_correlations_nt")
        grad_mod = importlib.import_module(oqupy_module.__name__ + ".gradient")
        grad_mod.compute_gradient_and_dynamics = _installed.pop("compute_gradient_and_dynamics")
        sd_mod.compute_dynamics_with_field = _installed.pop("compute_dynamics_with_field")
        pkg = _installed.pop("compute_dynamics_with_field_pkg", None)
        if pkg is not None:
            oqupy_module.compute_dynamics_with_field = pkg
        pkg = _installed.pop("compute_correlations_nt_pkg", None)
        if pkg is not None:
            oqupy_module.compute_correlations_nt = pkg
