"""Python side of the task API: ``StoppableTask`` over ``sbg_task`` and the
polling loop of ``stablebear/async_task.py:4-50``.

A task runs on a native worker thread; ``wait_for`` releases the GIL (ctypes
drops it for every foreign call), worker errors surface once from the call
that observes completion (``include/sbear/task.hpp:84-96``).
"""
from __future__ import annotations

import ctypes

from . import _native as nat


class StoppableTask:
    """Handle of one native task (the reference's ``StoppableTask_void``)."""

    def __init__(self, handle, keepalive=()):
        self._h = handle
        self._keep = tuple(keepalive)  # buffers the worker reads or writes

    def _handle(self):
        if self._h is None:
            raise RuntimeError("task already destroyed")
        return self._h

    def start(self):
        nat.check(nat.lib().sbg_task_start(self._handle()))
        return self

    def wait_for(self, ms: int) -> bool:
        fin = ctypes.c_int(0)
        st = nat.lib().sbg_task_wait_for(self._handle(), int(ms), ctypes.byref(fin))
        nat.check(st)
        return bool(fin.value)

    def wait(self):
        nat.check(nat.lib().sbg_task_wait(self._handle()))

    def request_stop(self):
        if self._h is not None:
            nat.lib().sbg_task_request_stop(self._h)

    def stop_requested(self) -> bool:
        return bool(self._h is not None and nat.lib().sbg_task_stop_requested(self._h))

    def _progress(self):
        t, c, s = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        nat.check(nat.lib().sbg_task_progress(self._handle(), ctypes.byref(t), ctypes.byref(c), ctypes.byref(s)))
        return t.value, c.value, s.value

    def work_total(self) -> int:
        return self._progress()[0]

    def work_completed(self) -> int:
        return self._progress()[1]

    def work_step(self) -> int:
        return self._progress()[2]

    def _text(self):
        d = ctypes.create_string_buffer(256)
        u = ctypes.create_string_buffer(64)
        nat.check(nat.lib().sbg_task_step_text(self._handle(), d, 256, u, 64))
        return d.value.decode(), u.value.decode()

    def work_step_desc(self) -> str:
        return self._text()[0]

    def work_step_unit(self) -> str:
        return self._text()[1]

    def close(self):
        if self._h is not None:
            nat.lib().sbg_task_destroy(self._h)
            self._h = None
            self._keep = ()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class EmptyTask:
    """A task that is already finished (``include/sbear/task.hpp:174-192``)."""

    def start(self):
        return self

    def wait_for(self, ms: int) -> bool:
        return True

    def wait(self):
        return None

    def request_stop(self):
        return None

    def stop_requested(self) -> bool:
        return False

    def work_total(self) -> int:
        return 0

    def work_completed(self) -> int:
        return 0

    def work_step(self) -> int:
        return 0

    def work_step_desc(self) -> str:
        return ""

    def work_step_unit(self) -> str:
        return ""

    def close(self):
        return None


def _make_progress(task):
    try:
        from tqdm import tqdm
    except ImportError:  # tqdm is optional
        return None
    return tqdm(total=task.work_total(), unit_scale=True, unit=task.work_step_unit(), desc=task.work_step_desc())


def _wait_for_task(task, verbose=True):
    progress = _make_progress(task) if verbose else None
    work_step = task.work_step() if verbose else 0
    while not task.wait_for(50):
        if progress is not None:
            progress.update(task.work_completed() - progress.n)
            step = task.work_step()
            if step != work_step:
                work_step = step
                progress = _make_progress(task)
    if progress is not None:
        progress.update(task.work_completed() - progress.n)


def _run_task(task_fn, verbose=True):
    """Poll a task to completion; on any exit (including KeyboardInterrupt)
    request a stop and drain it (stablebear/async_task.py:32-50)."""
    task = None
    try:
        task = task_fn()
        _wait_for_task(task, verbose=verbose)
    finally:
        if task is not None:
            task.request_stop()
            try:
                _wait_for_task(task, verbose=False)
            except BaseException:
                pass
            task.close()
