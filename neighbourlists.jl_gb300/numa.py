"""Placement of pinned host buffers on the host's NUMA nodes.

End-to-end use copies every pair array between the GPU and pinned host
memory.  On a multi-socket host (a Grace pair: each Grace has its own memory
and its own link to its GPUs) a buffer on the far node crosses the
socket-to-socket link as well.  These helpers find the GPU's own node,
allocate pinned buffers there (the allocating thread is bound to that node's
CPUs, so the pages are placed locally by first touch), and report which node
a buffer's pages are on (the kernel's move_pages in query mode).  Linux only;
every function degrades to "unknown" (None) elsewhere.
"""
from __future__ import annotations

import ctypes
import os
import platform
from typing import Dict, Optional, Set

import torch

_SYS_MOVE_PAGES = {"x86_64": 279, "aarch64": 239}


def gpu_numa_node(device=None) -> Optional[int]:
    """NUMA node of the CPUs nearest the GPU (sysfs numa_node of its PCI
    device); None when the host does not say."""
    dev = torch.device(device if device is not None else "cuda")
    try:
        props = torch.cuda.get_device_properties(dev)
        bus = "%04x:%02x:%02x.0" % (props.pci_domain_id, props.pci_bus_id, props.pci_device_id)
        with open(f"/sys/bus/pci/devices/{bus}/numa_node") as f:
            node = int(f.read().strip())
        return node if node >= 0 else None
    except (OSError, ValueError, AttributeError, RuntimeError, AssertionError):
        return None


def node_cpus(node: int) -> Set[int]:
    """CPUs of a NUMA node (empty for a node without CPUs, e.g. GPU memory)."""
    try:
        with open(f"/sys/devices/system/node/node{node}/cpulist") as f:
            text = f.read().strip()
    except OSError:
        return set()
    cpus: Set[int] = set()
    for part in filter(None, text.split(",")):
        a, _, b = part.partition("-")
        cpus.update(range(int(a), int(b or a) + 1))
    return cpus


def cpu_nodes() -> Dict[int, Set[int]]:
    """Every NUMA node that has CPUs, with its CPUs."""
    out: Dict[int, Set[int]] = {}
    try:
        names = os.listdir("/sys/devices/system/node")
    except OSError:
        return out
    for n in names:
        if n.startswith("node") and n[4:].isdigit():
            c = node_cpus(int(n[4:]))
            if c:
                out[int(n[4:])] = c
    return out


def pinned_on_node(shape, dtype, node: Optional[int]) -> torch.Tensor:
    """A pinned host tensor whose pages are placed on ``node`` (first touch by
    a thread bound to the node's CPUs); an ordinary pinned tensor when the
    node is unknown or has no CPUs."""
    cpus = node_cpus(node) if node is not None else set()
    if not cpus or not hasattr(os, "sched_setaffinity"):
        return torch.empty(shape, dtype=dtype).pin_memory()
    old = os.sched_getaffinity(0)
    try:
        os.sched_setaffinity(0, cpus)
        t = torch.empty(shape, dtype=dtype)
        t.zero_()  # first touch on the node
        return t.pin_memory()  # the pinned copy is allocated and filled here as well
    finally:
        os.sched_setaffinity(0, old)


def page_nodes(t: torch.Tensor, samples: int = 64) -> Dict[int, int]:
    """Node of a sample of the tensor's pages (move_pages query mode):
    {node: pages}; {} when the query is not available."""
    nr = _SYS_MOVE_PAGES.get(platform.machine())
    if nr is None or t.numel() == 0:
        return {}
    try:
        libc = ctypes.CDLL(None, use_errno=True)
        page = os.sysconf("SC_PAGE_SIZE")
        base = t.data_ptr() // page * page
        end = t.data_ptr() + t.numel() * t.element_size()
        npages = max((end - base) // page, 1)
        step = max(npages // samples, 1)
        addrs = [base + k * step * page for k in range(min(samples, npages))]
        n = len(addrs)
        pages = (ctypes.c_void_p * n)(*addrs)
        status = (ctypes.c_int * n)()
        r = libc.syscall(ctypes.c_long(nr), ctypes.c_int(0), ctypes.c_ulong(n), pages, None, status, ctypes.c_int(0))
        if r != 0:
            return {}
        out: Dict[int, int] = {}
        for s in status:
            if s >= 0:
                out[s] = out.get(s, 0) + 1
        return out
    except (OSError, AttributeError, ValueError):
        return {}
