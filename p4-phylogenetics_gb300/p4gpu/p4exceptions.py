"""Exceptions, mirroring p4/p4exceptions.py (P4Error carries a message list)."""


class P4Error(Exception):
    def __init__(self, msg=""):
        if isinstance(msg, (list, tuple)):
            msg = "\n".join(str(m) for m in msg)
        Exception.__init__(self, msg)
        self.msg = msg
