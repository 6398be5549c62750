"""Oracle continuation schedules (TEST INFRASTRUCTURE).

Restates scikit-topt/sktopt/tools/scheduler.py: the schedule functions
44-261 and ``Scheduler.value`` 809-830 (``iters_max`` is the optimizer's
``max_iters``; a schedule with no ``num_steps`` returns its target).
"""
from __future__ import annotations


def schedule_constant(it, total, target_value=0.4, **_):
    return target_value


def schedule_step(it, total, initial_value=1.0, target_value=0.4,
                  num_steps=10, **_):
    if total <= 0:
        raise ValueError("total must be positive")
    if num_steps <= 1:
        return target_value
    step_length = total / num_steps
    step_index = min(int(it // step_length), num_steps - 1)
    alpha = step_index / (num_steps - 1)
    return (1 - alpha) * initial_value + alpha * target_value


def schedule_step_accelerating(it, total, initial_value=1.0, target_value=0.4,
                               num_steps=10, curvature=3.0, **_):
    if total <= 0:
        raise ValueError("total must be positive")
    if num_steps <= 1:
        return target_value
    step_length = total / num_steps
    step_index = min(int(it // step_length), num_steps - 1)
    alpha = step_index / (num_steps - 1)
    a = alpha ** curvature
    return (1 - a) * initial_value + a * target_value


def schedule_step_decelerating(it, total, initial_value=1.0, target_value=0.4,
                               num_steps=10, curvature=3.0, **_):
    if total <= 0:
        raise ValueError("total must be positive")
    if num_steps <= 1:
        return target_value
    step_length = total / num_steps
    step_index = min(int(it // step_length), num_steps - 1)
    alpha = step_index / (num_steps - 1)
    a = 1 - (1 - alpha) ** curvature
    return (1 - a) * initial_value + a * target_value


def schedule_sawtooth_decay(it, total, initial_value=0.1, target_value=0.05,
                            num_steps=6, **_):
    if total <= 0 or num_steps <= 0:
        raise ValueError("total and num_steps must be positive")
    it0 = it - 1
    step_size = total / num_steps
    step_index = int(it0 // step_size)
    local_index = it0 - step_index * step_size
    alpha = min(local_index / step_size, 1.0)
    return (1 - alpha) * initial_value + alpha * target_value


FUNCS = {
    "Constant": schedule_constant,
    "ConstantOne": schedule_constant,
    "Step": schedule_step,
    "StepToOne": schedule_step,
    "StepAccelerating": schedule_step_accelerating,
    "StepAcceleratingToOne": schedule_step_accelerating,
    "StepDecelerating": schedule_step_decelerating,
    "StepDeceleratingToOne": schedule_step_decelerating,
    "SawtoothDecay": schedule_sawtooth_decay,
    "None": None,
}


def value(kind, it, iters_max, init=None, target=None, num_steps=None,
          curvature=None):
    """Scheduler.value scheduler.py:809-830 after ``from_config`` 747-807."""
    if kind in ("Constant",):
        init, num_steps = target, None
    if kind == "ConstantOne":
        init = target = 1.0
        num_steps = None
    if kind in ("StepToOne", "StepAcceleratingToOne", "StepDeceleratingToOne"):
        target = 1.0
        if num_steps:
            init = 1.0 / num_steps
    if target is None:
        return None
    if num_steps is None or num_steps < 0:
        return target
    if it >= iters_max:
        return target
    return FUNCS[kind](it=it, total=iters_max, initial_value=init,
                       target_value=target, num_steps=num_steps,
                       curvature=curvature)
