set output "hist_sp_MOTIF00002.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-32.6689:14.394]
set yrange [0:6774]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_sp_MOTIF00002.dat" using 1:2 title 'MOTIF00002 (sp)' with boxes
