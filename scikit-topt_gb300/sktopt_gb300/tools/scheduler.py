"""Continuation schedules (host scalars per iteration).

Same configuration surface and values as sktopt/tools/scheduler.py:
``SchedulerConfig`` factories (273-682), ``Scheduler.from_config`` /
``value`` (747-830), the schedule functions (14-261) and ``Schedulers``
(1152-1281, without the matplotlib export).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Callable, Literal, Optional


def _step_index(it, total, num_steps):
    if total <= 0:
        raise ValueError("total must be positive")
    return min(int(it // (total / num_steps)), num_steps - 1)


def schedule_constant(it, total, target_value=0.4, **_):
    return target_value


def schedule_step(it, total, initial_value=1.0, target_value=0.4, num_steps=10, **_):
    if total <= 0:
        raise ValueError("total must be positive")
    if num_steps <= 1:
        return target_value
    a = _step_index(it, total, num_steps) / (num_steps - 1)
    return (1 - a) * initial_value + a * target_value


def schedule_step_accelerating(it, total, initial_value=1.0, target_value=0.4,
                               num_steps=10, curvature=3.0, **_):
    if total <= 0:
        raise ValueError("total must be positive")
    if num_steps <= 1:
        return target_value
    a = (_step_index(it, total, num_steps) / (num_steps - 1)) ** curvature
    return (1 - a) * initial_value + a * target_value


def schedule_step_decelerating(it, total, initial_value=1.0, target_value=0.4,
                               num_steps=10, curvature=3.0, **_):
    if total <= 0:
        raise ValueError("total must be positive")
    if num_steps <= 1:
        return target_value
    a = 1 - (1 - _step_index(it, total, num_steps) / (num_steps - 1)) ** curvature
    return (1 - a) * initial_value + a * target_value


def schedule_sawtooth_decay(it, total, initial_value=0.1, target_value=0.05, num_steps=6,
                            **_):
    if total <= 0 or num_steps <= 0:
        raise ValueError("total and num_steps must be positive")
    size = total / num_steps
    k = (it - 1) - int((it - 1) // size) * size
    a = min(k / size, 1.0)
    return (1 - a) * initial_value + a * target_value


_TO_ONE = ("StepToOne", "StepAcceleratingToOne", "StepDeceleratingToOne")
_FUNCS = {
    "Constant": schedule_constant, "ConstantOne": schedule_constant,
    "Step": schedule_step, "StepToOne": schedule_step,
    "StepAccelerating": schedule_step_accelerating,
    "StepAcceleratingToOne": schedule_step_accelerating,
    "StepDecelerating": schedule_step_decelerating,
    "StepDeceleratingToOne": schedule_step_decelerating,
    "SawtoothDecay": schedule_sawtooth_decay, "None": None,
}


@dataclass
class SchedulerConfig:
    name: Optional[str] = None
    init_value: Optional[float] = None
    target_value: Optional[float] = None
    num_steps: Optional[int] = None
    iters_max: Optional[int] = None
    curvature: Optional[float] = None
    scheduler_type: Literal["Constant", "ConstantOne", "Step", "StepAccelerating",
                            "StepDecelerating", "SawtoothDecay", "StepToOne",
                            "StepAcceleratingToOne", "StepDeceleratingToOne",
                            "None"] = "Constant"

    @classmethod
    def from_defaults(cls, name=None, init_value=None, target_value=None, num_steps=None,
                      iters_max=None, curvature=None, scheduler_type="Constant"):
        t = scheduler_type
        if t == "Constant":
            if target_value is None:
                raise ValueError("Should set target_value")
            if init_value is None:
                init_value = target_value
        elif t == "ConstantOne":
            init_value = target_value = 1.0
        elif t in _TO_ONE:
            if num_steps is None:
                raise ValueError("Should set num_steps")
            if num_steps <= 0:
                raise ValueError(f"num_steps must be positive for {t}")
            if t != "StepToOne" and curvature is None:
                raise ValueError("Should set curvature")
            if target_value is not None and not math.isclose(target_value, 1.0):
                raise ValueError(f"{t} fixes target_value to 1.0")
            target_value, init_value = 1.0, 1.0 / num_steps
        elif t in ("Step", "StepAccelerating", "StepDecelerating", "SawtoothDecay"):
            for v, nm in ((init_value, "init_value"), (target_value, "target_value"),
                          (num_steps, "num_steps")):
                if v is None:
                    raise ValueError(f"Should set {nm}")
            if t in ("StepAccelerating", "StepDecelerating") and curvature is None:
                raise ValueError("Should set curvature")
        elif t != "None":
            raise ValueError(f"unknown scheduler_type {t}")
        return cls(name, init_value, target_value, num_steps, iters_max, curvature, t)

    @classmethod
    def none(cls):
        return cls.from_defaults(scheduler_type="None")

    @classmethod
    def constant(cls, name=None, target_value=1.0):
        return cls.from_defaults(name, target_value, target_value, None, None, None,
                                 "Constant")

    @classmethod
    def constant_one(cls, name=None):
        return cls.from_defaults(name, 1.0, 1.0, None, None, None, "ConstantOne")

    @classmethod
    def step(cls, name=None, init_value=None, target_value=None, num_steps=None,
             iters_max=None):
        return cls.from_defaults(name, init_value, target_value, num_steps, iters_max, None,
                                 "Step")

    @classmethod
    def step_to_one(cls, name=None, num_steps=None, iters_max=None):
        return cls.from_defaults(name, None, 1.0, num_steps, iters_max, None, "StepToOne")

    @classmethod
    def step_accelerating(cls, name=None, init_value=None, target_value=None,
                          num_steps=None, iters_max=None, curvature=None):
        return cls.from_defaults(name, init_value, target_value, num_steps, iters_max,
                                 curvature, "StepAccelerating")

    @classmethod
    def step_accelerating_to_one(cls, name=None, num_steps=None, iters_max=None,
                                 curvature=None):
        return cls.from_defaults(name, None, 1.0, num_steps, iters_max, curvature,
                                 "StepAcceleratingToOne")

    @classmethod
    def step_decelerating(cls, name=None, init_value=None, target_value=None,
                          num_steps=None, iters_max=None, curvature=None):
        return cls.from_defaults(name, init_value, target_value, num_steps, iters_max,
                                 curvature, "StepDecelerating")

    @classmethod
    def step_decelerating_to_one(cls, name=None, num_steps=None, iters_max=None,
                                 curvature=None):
        return cls.from_defaults(name, None, 1.0, num_steps, iters_max, curvature,
                                 "StepDeceleratingToOne")

    @classmethod
    def sawtooth_decay(cls, name=None, init_value=0.1, target_value=0.05, iters_max=100,
                       num_steps=6):
        return cls(name, init_value, target_value, num_steps, iters_max, None,
                   "SawtoothDecay")


class Scheduler:
    def __init__(self, name, init_value, target_value, num_steps=None, iters_max=None,
                 curvature=None, func: Callable | None = schedule_step):
        self.name = name
        self.init_value = init_value
        self.target_value = target_value
        self.num_steps = num_steps
        self.iters_max = iters_max
        self.curvature = curvature
        self.func = func

    @classmethod
    def from_config(cls, cfg: SchedulerConfig):
        t = cfg.scheduler_type
        if t not in _FUNCS:
            raise ValueError(f"{t} not in {list(_FUNCS)}")
        if t in ("Constant", "ConstantOne"):
            if t == "ConstantOne":
                cfg.target_value = 1.0
            cfg.init_value = cfg.target_value
            cfg.iters_max = cfg.num_steps = cfg.curvature = None
        elif t in _TO_ONE:
            cfg.target_value = 1.0
            if cfg.num_steps:
                cfg.init_value = 1.0 / cfg.num_steps
        return cls(cfg.name, cfg.init_value, cfg.target_value, cfg.num_steps,
                   iters_max=cfg.iters_max, curvature=cfg.curvature, func=_FUNCS[t])

    def value(self, it):
        if self.target_value is None:
            return None
        if self.num_steps is None or (isinstance(self.num_steps, (int, float))
                                      and self.num_steps < 0):
            return self.target_value
        if it >= self.iters_max:
            return self.target_value
        return self.func(it=it, total=self.iters_max, initial_value=self.init_value,
                         target_value=self.target_value, num_steps=self.num_steps,
                         curvature=self.curvature)


class Schedulers:
    def __init__(self, dst_path: str = "."):
        self.scheduler_list: list[Scheduler] = []
        self.dst_path = dst_path

    def set_iters_max(self, iters_max: int):
        for s in self.scheduler_list:
            s.iters_max = iters_max

    def add_object(self, s: Scheduler):
        self.scheduler_list.append(s)

    def add_object_from_config(self, cfg: SchedulerConfig, rewrite_name: str | None):
        if isinstance(rewrite_name, str):
            cfg.name = rewrite_name
        self.add_object(Scheduler.from_config(cfg))

    def add(self, name, init_value, target_value, num_steps, iters_max=None, curvature=None,
            func=schedule_step):
        self.scheduler_list.append(Scheduler(name, init_value, target_value, num_steps,
                                             iters_max, curvature=curvature, func=func))

    def values_as_dict(self, it):
        return {s.name: s.value(it) for s in self.scheduler_list}

    def values_as_list(self, it, order, export_log=False, precision=4):
        d = self.values_as_dict(it)
        return [d[k] for k in order]

    def value_on_a_scheduler(self, key, it):
        return self.values_as_list(it, [key])[0]
