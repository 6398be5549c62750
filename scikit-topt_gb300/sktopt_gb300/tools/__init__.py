from .scheduler import (SchedulerConfig, Scheduler, Schedulers, schedule_step,
                        schedule_step_accelerating, schedule_step_decelerating,
                        schedule_sawtooth_decay, schedule_constant)
from .history import HistoryCollection

__all__ = ["SchedulerConfig", "Scheduler", "Schedulers", "HistoryCollection",
           "schedule_step", "schedule_step_accelerating", "schedule_step_decelerating",
           "schedule_sawtooth_decay", "schedule_constant"]
