"""Cancel-token shapes that big-wave's history, checkpoint and detector steps are given, built the
same way by the fixture generator (make_token_golden.py) and by the tests."""
from __future__ import annotations

import threading


class _Obj:
    pass


def _attrs(**kw):
    o = _Obj()
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class _ProgressAndEvent:
    """A 3-argument progress callback that also carries an `is_set` attribute."""
    is_set = True

    def __call__(self, stage, done, total):
        return None


class _ZeroArgCallableWithAttr:
    is_set = True

    def __call__(self):
        return False


class _MethodToken:
    def __init__(self, answer):
        self._answer = answer

    def is_cancelled(self):
        return self._answer


def _event(set_it: bool):
    e = threading.Event()
    if set_it:
        e.set()
    return e


CASES = {
    "none": lambda: None,
    "bool_true": lambda: True,
    "bool_false": lambda: False,
    "callable_true": lambda: (lambda: True),
    "callable_false": lambda: (lambda: False),
    "attr_is_set_true": lambda: _attrs(is_set=True),
    "attr_is_set_false": lambda: _attrs(is_set=False),
    "attr_is_set_none_then_cancelled_true": lambda: _attrs(is_set=None, cancelled=True),
    "attr_cancelled_true": lambda: _attrs(cancelled=True),
    "attr_is_cancelled_zero": lambda: _attrs(is_cancelled=0),
    "method_is_cancelled_true": lambda: _MethodToken(True),
    "method_is_cancelled_false": lambda: _MethodToken(False),
    "event_set": lambda: _event(True),
    "event_clear": lambda: _event(False),
    "progress_callback_with_is_set": lambda: _ProgressAndEvent(),
    "zero_arg_callable_with_is_set": lambda: _ZeroArgCallableWithAttr(),
    "plain_object": lambda: _Obj(),
    "int_one": lambda: 1,
}


def outcome(fn, token) -> str:
    """'True' / 'False', or the name of the exception the check raised."""
    try:
        return str(bool(fn(token)))
    except Exception as exc:  # noqa: BLE001 - the exception type is the recorded answer
        return type(exc).__name__
