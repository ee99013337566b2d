set output "hist_sp_MOTIF00004.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-59.7532:21.2064]
set yrange [0:8444]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_sp_MOTIF00004.dat" using 1:2 title 'MOTIF00004 (sp)' with boxes
