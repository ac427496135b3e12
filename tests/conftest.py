'''Shared test setup: the `gpu` marker, the repository root on the import path, and a seeded torch
generator before every test (as the reference's tests/conftest.py:7-10 seeds it).'''
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA device (a GB300) and the built extension')


@pytest.fixture(autouse = True)
def seed_generator():
    import torch
    torch.manual_seed(0)
