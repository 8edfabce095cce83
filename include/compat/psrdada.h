// Drop-in replacement for psrdada/include/psrdada.h (header-only).
//
// PSRDADA file reader with the reference's interface (psrdada.h:16-43,
// psrdada.cpp:3-127): a 4096-byte ASCII header (BW, FREQ, NBIT, NCHAN, NDIM,
// NPOL, one "KEY value" per line), then frames of 2048 samples per polarisation,
// polarisations interleaved frame by frame.  NBIT 16 reads uint16_pair samples
// into pol1_in/pol2_in as the reference does; NBIT 8 (new) reads int8 I/Q pairs
// into pol1_i8/pol2_i8 (2 bytes per sample) for processors initialised with
// MSOSM_IN_I8.  Unlike the reference, failures throw std::runtime_error instead
// of calling exit(1), and short reads are reported by readSamples()'s return.
#pragma once
#include "globals.h"
#include <sstream>
#include <stdexcept>
#include <utility>

auto constexpr blockSize = 4096;
auto constexpr frameSamples = 2048;

class PSRDADA
{
  public:
    explicit PSRDADA(string filename)
    {
        infileName = filename;
        infile.open(filename, ios::binary | ios::ate);
        if (!infile.is_open())
            throw std::runtime_error("Cannot open file: " + filename);
        filesize = (unsigned long)infile.tellg();
        infile.seekg(0, ios::beg);
        outfileName = filename.substr(0, filename.find_last_of('.')) + "_dedisp_folded.txt";
        if (filesize < (unsigned long)blockSize)
            throw std::runtime_error("file shorter than the 4096-byte header: " + filename);
        infile.read(headerBuffer, blockSize);
        string header(headerBuffer, blockSize);
        header.erase(std::remove(header.begin(), header.end(), '\0'), header.end());
        istringstream iss(header);
        string ln;
        while (getline(iss, ln))
        {
            auto kv = split(ln);
            try
            {
                if (kv.first == "BW")
                    bw = stof(kv.second);
                else if (kv.first == "FREQ")
                    fc = stof(kv.second);
                else if (kv.first == "NBIT")
                    nbit = stoi(kv.second);
                else if (kv.first == "NCHAN")
                    nchan = stoi(kv.second);
                else if (kv.first == "NDIM")
                    ndim = stoi(kv.second);
                else if (kv.first == "NPOL")
                    npol = stoi(kv.second);
            }
            catch (const std::exception &)
            {
                throw std::runtime_error("bad header value for " + kv.first);
            }
        }
        if (verbose)
        {
            cout << "Bandwidth: " << bw << " MHz" << endl;
            cout << "Center frequency: " << fc << " MHz" << endl;
            cout << "Data precision: " << nbit << " bit" << endl;
            cout << "Polarization number: " << npol << endl;
        }
    }
    ~PSRDADA()
    {
        infile.close();
        delete[] pol1_in;
        delete[] pol2_in;
        delete[] pol1_i8;
        delete[] pol2_i8;
    }
    size_t sample_bytes() const { return nbit == 8 ? 2 : sizeof(uint16_pair); }
    void initBuffer(size_t n)
    {
        if (n % frameSamples != 0)
            throw std::runtime_error("n must be a multiple of frameSamples (2048)");
        if (npol != 1 && npol != 2)
            throw std::runtime_error("Unsupported polarization number: " + to_string(npol));
        if (nbit != 16 && nbit != 8)
            throw std::runtime_error("Unsupported NBIT: " + to_string(nbit));
        if (nbit == 16)
        {
            pol1_in = new uint16_pair[n];
            pol2_in = new uint16_pair[n];
        }
        else
        {
            pol1_i8 = new int8_t[2 * n];
            pol2_i8 = new int8_t[2 * n];
        }
        frameCount = (int)(n / frameSamples);
        readCount = (unsigned long)((filesize - blockSize) / (npol * n * sample_bytes()));
    }
    // Reads frameCount frames per polarisation; false on a short read.
    bool readSamples()
    {
        const size_t fb = frameSamples * sample_bytes();
        char *p1 = nbit == 16 ? (char *)pol1_in : (char *)pol1_i8;
        char *p2 = nbit == 16 ? (char *)pol2_in : (char *)pol2_i8;
        for (int i = 0; i < frameCount; i++)
        {
            if (!infile.read(p1 + i * fb, fb))
                return false;
            if (npol == 2 && !infile.read(p2 + i * fb, fb))
                return false;
        }
        return true;
    }

  public:
    char headerBuffer[blockSize];
    ifstream infile;
    string infileName;
    unsigned long filesize = 0;
    unsigned long readCount = 0;
    string outfileName;
    float bw = 0, fc = 0;
    int nbit = 16, nchan = 1, ndim = 2, npol = 1;
    int hdr_size = blockSize;
    uint16_pair *pol1_in = nullptr;
    uint16_pair *pol2_in = nullptr;
    int8_t *pol1_i8 = nullptr;
    int8_t *pol2_i8 = nullptr;
    int frameCount = 0;

  private:
    static pair<string, string> split(const string &input)
    {
        size_t pos = input.find_first_of(" \t");
        if (pos == string::npos)
            return {input, ""};
        size_t start = input.find_first_not_of(" \t", pos);
        if (start == string::npos)
            return {input.substr(0, pos), ""};
        return {input.substr(0, pos), input.substr(start)};
    }
};
